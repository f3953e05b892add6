/*
 * uwo_solve.c -- CPU Stokes assembly and BSSCR solve (TEST INFRASTRUCTURE and
 * the timed CPU baseline).  Plain C + OpenMP, FP64.
 *
 * The reference solves with PETSc (BSSCR_DRIVER_auglag,
 * L/Solvers/KSPSolvers/src/BSSCR/auglag-driver-DGTGD.c:64-578: velocity
 * pre-solve, Schur-complement pressure solve preconditioned by the assembled
 * Uzawa term, velocity back-solve; FGMRES + geometric multigrid inside).
 * PETSc is not available, so this file runs the same BSSCR structure with the
 * same kernels as the GPU library (matrix-free viscous operator from exact
 * equivalent-quadrature weights, multigrid-preconditioned CG for velocity,
 * right-preconditioned FGMRES on the Schur complement), on host cores.
 *
 *   L/ = src/underworld/libUnderworld/
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#define MAXLEV 16

typedef struct {
    int res[3];
    int64_t n_el, n_nodes, n_dof;
    double* ax[3];
    double* W;        /* [nq][n_el] */
    uint8_t* bc;      /* [n_dof] */
    double* diag;
    double lmax;
    double* cinv;     /* dense inverse on the coarsest level */
    double *r, *d, *t, *b, *x;
} lev_t;

typedef struct {
    int dim, nq, nlev;
    int64_t nv, np;
    lev_t L[MAXLEV];
    double *f, *h, *shat, *bcval;
    /* solver vectors */
    double *cg_r, *cg_z, *cg_p, *cg_q, *u1, *u2, *ftil, *bvec, *hhat, *pt1, *pt2;
    double **V, **Z;
    int restart;
} uwo_sys;

static double* dalloc(int64_t n) { return (double*)calloc((size_t)(n > 0 ? n : 1), sizeof(double)); }

uwo_sys* uwo_sys_create(int dim, const int* res, const double* ax0, const double* ax1, const double* ax2) {
    uwo_sys* s = (uwo_sys*)calloc(1, sizeof(uwo_sys));
    const double* ax[3] = {ax0, ax1, ax2};
    s->dim = dim;
    s->nq = dim == 3 ? 27 : 9;
    int r[3] = {res[0], res[1], dim == 3 ? res[2] : 1};
    int nlev = 1;
    {
        int q[3] = {r[0], r[1], r[2]};
        while (nlev < MAXLEV) {
            int even = 1;
            for (int i = 0; i < dim; i++) even = even && (q[i] % 2 == 0);
            if (!even) break;
            for (int i = 0; i < dim; i++) q[i] /= 2;
            nlev++;
        }
    }
    s->nlev = nlev;
    for (int l = 0; l < nlev; l++) {
        lev_t* L = &s->L[l];
        L->n_el = 1; L->n_nodes = 1;
        for (int i = 0; i < 3; i++) {
            L->res[i] = i < dim ? (r[i] >> l) : 1;
            L->n_el *= L->res[i];
            if (i < dim) L->n_nodes *= L->res[i] + 1;
            if (i < dim) {
                L->ax[i] = dalloc(L->res[i] + 1);
                for (int k = 0; k <= L->res[i]; k++) L->ax[i][k] = ax[i][(size_t)k << l];
            }
        }
        L->n_dof = L->n_nodes * dim;
        L->W = dalloc(s->nq * L->n_el);
        L->bc = (uint8_t*)calloc((size_t)L->n_dof, 1);
        L->diag = dalloc(L->n_dof);
        L->r = dalloc(L->n_dof); L->d = dalloc(L->n_dof); L->t = dalloc(L->n_dof);
        L->b = dalloc(L->n_dof); L->x = dalloc(L->n_dof);
        if (l == nlev - 1) L->cinv = dalloc(L->n_dof * L->n_dof);
    }
    s->nv = s->L[0].n_dof;
    s->np = s->L[0].n_el;
    s->f = dalloc(s->nv); s->h = dalloc(s->np); s->shat = dalloc(s->np); s->bcval = dalloc(s->nv);
    s->cg_r = dalloc(s->nv); s->cg_z = dalloc(s->nv); s->cg_p = dalloc(s->nv); s->cg_q = dalloc(s->nv);
    s->u1 = dalloc(s->nv); s->u2 = dalloc(s->nv); s->ftil = dalloc(s->nv); s->bvec = dalloc(s->nv);
    s->hhat = dalloc(s->np); s->pt1 = dalloc(s->np); s->pt2 = dalloc(s->np);
    s->restart = 30;
    s->V = (double**)calloc(s->restart + 1, sizeof(double*));
    s->Z = (double**)calloc(s->restart, sizeof(double*));
    for (int i = 0; i <= s->restart; i++) s->V[i] = dalloc(s->np);
    for (int i = 0; i < s->restart; i++) s->Z[i] = dalloc(s->np);
    return s;
}

void uwo_sys_destroy(uwo_sys* s) {
    if (!s) return;
    for (int l = 0; l < s->nlev; l++) {
        lev_t* L = &s->L[l];
        for (int i = 0; i < 3; i++) free(L->ax[i]);
        free(L->W); free(L->bc); free(L->diag); free(L->r); free(L->d); free(L->t); free(L->b); free(L->x);
        free(L->cinv);
    }
    free(s->f); free(s->h); free(s->shat); free(s->bcval);
    free(s->cg_r); free(s->cg_z); free(s->cg_p); free(s->cg_q); free(s->u1); free(s->u2);
    free(s->ftil); free(s->bvec); free(s->hhat); free(s->pt1); free(s->pt2);
    for (int i = 0; i <= s->restart; i++) free(s->V[i]);
    for (int i = 0; i < s->restart; i++) free(s->Z[i]);
    free(s->V); free(s->Z);
    free(s);
}

static void elem(const uwo_sys* s, const lev_t* L, int64_t e, int64_t* nodes, double* h) {
    int ex = (int)(e % L->res[0]), ey = (int)((e / L->res[0]) % L->res[1]);
    int ez = s->dim == 3 ? (int)(e / ((int64_t)L->res[0] * L->res[1])) : 0;
    h[0] = L->ax[0][ex + 1] - L->ax[0][ex];
    h[1] = L->ax[1][ey + 1] - L->ax[1][ey];
    h[2] = s->dim == 3 ? L->ax[2][ez + 1] - L->ax[2][ez] : 1.0;
    int64_t nx = L->res[0] + 1, ny = L->res[1] + 1;
    int nn = s->dim == 3 ? 8 : 4;
    for (int n = 0; n < nn; n++) {
        int i = n & 1, j = (n >> 1) & 1, k = (n >> 2) & 1;
        nodes[n] = (ex + i) + nx * ((ey + j) + ny * (int64_t)(ez + k));
    }
}

static double lderiv(int dim, int n, int d, const int* pt) {
    double v = 1.0;
    for (int e = 0; e < dim; e++) {
        int sg = (n >> e) & 1;
        if (e == d) v *= sg ? 0.5 : -0.5;
        else v *= (pt[e] == 1) ? 0.5 : ((pt[e] == 2) == (sg == 1) ? 1.0 : 0.0);
    }
    return v;
}

/* Equivalent-quadrature weights and the body-force vector from the PIC points
 * (the CPU twin of libuwg's assembly).  Slot order: cell tables in CSR. */
void uwo_sys_assemble_points(uwo_sys* s, const int32_t* off, const int32_t* lst, const double* ip_xi,
                             const double* ip_w, const double* eta, const double* body) {
    lev_t* L = &s->L[0];
    int dim = s->dim, nq = s->nq, nen = dim == 3 ? 8 : 4;
    memset(s->f, 0, sizeof(double) * s->nv);
    /* element loop; force scatter with a per-colour schedule to stay race free */
    for (int color = 0; color < (1 << dim); color++) {
#pragma omp parallel for schedule(static)
        for (int64_t e = 0; e < L->n_el; e++) {
            int ex = (int)(e % L->res[0]), ey = (int)((e / L->res[0]) % L->res[1]);
            int ez = dim == 3 ? (int)(e / ((int64_t)L->res[0] * L->res[1])) : 0;
            int col = (ex & 1) | ((ey & 1) << 1) | ((ez & 1) << 2);
            if (col != color) continue;
            int64_t nodes[8];
            double h[3], Wl[27] = {0}, fe[24] = {0};
            elem(s, L, e, nodes, h);
            double detJ = dim == 3 ? (h[0] * 0.5) * (h[1] * 0.5) * (h[2] * 0.5) : (h[0] * 0.5) * (h[1] * 0.5);
            for (int32_t q = off[e]; q < off[e + 1]; q++) {
                int32_t p = lst[q];
                double l[3][3];
                for (int d = 0; d < 3; d++) {
                    double x = d < dim ? ip_xi[(int64_t)q * dim + d] : 0.0;
                    l[d][0] = 0.5 * x * (x - 1.0); l[d][1] = 1.0 - x * x; l[d][2] = 0.5 * x * (x + 1.0);
                    if (d >= dim) { l[d][0] = 1.0; l[d][1] = 0.0; l[d][2] = 0.0; }
                }
                double wd = ip_w[q] * detJ, c = eta[p] * wd;
                for (int kz = 0; kz < (dim == 3 ? 3 : 1); kz++)
                    for (int ky = 0; ky < 3; ky++)
                        for (int kx = 0; kx < 3; kx++) Wl[kx + 3 * ky + 9 * kz] += c * l[0][kx] * l[1][ky] * l[2][kz];
                if (body) {
                    for (int n = 0; n < nen; n++) {
                        double N = 1.0;
                        for (int d = 0; d < dim; d++) {
                            double sg = ((n >> d) & 1) ? 1.0 : -1.0;
                            N *= 0.5 * (1.0 + sg * ip_xi[(int64_t)q * dim + d]);
                        }
                        for (int i = 0; i < dim; i++) fe[n * dim + i] += wd * body[(int64_t)p * dim + i] * N;
                    }
                }
            }
            for (int j = 0; j < nq; j++) L->W[(int64_t)j * L->n_el + e] = Wl[j];
            for (int n = 0; n < nen; n++)
                for (int i = 0; i < dim; i++) s->f[nodes[n] * dim + i] += fe[n * dim + i];
        }
    }
}

/* y = P K P x + (I - P) x, element colouring instead of atomics */
static void applyK(const uwo_sys* s, int l, const double* x, double* y) {
    const lev_t* L = &s->L[l];
    int dim = s->dim, nq = s->nq, nen = dim == 3 ? 8 : 4;
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < L->n_dof; i++) y[i] = L->bc[i] ? x[i] : 0.0;
    for (int color = 0; color < (1 << dim); color++) {
#pragma omp parallel for schedule(static)
        for (int64_t e = 0; e < L->n_el; e++) {
            int ex = (int)(e % L->res[0]), ey = (int)((e / L->res[0]) % L->res[1]);
            int ez = dim == 3 ? (int)(e / ((int64_t)L->res[0] * L->res[1])) : 0;
            int col = (ex & 1) | ((ey & 1) << 1) | ((ez & 1) << 2);
            if (col != color) continue;
            int64_t nodes[8];
            double h[3], u[8][3], out[8][3];
            elem(s, L, e, nodes, h);
            double hi[3] = {2.0 / h[0], 2.0 / h[1], 2.0 / h[2]};
            for (int n = 0; n < nen; n++)
                for (int c = 0; c < dim; c++) {
                    int64_t dof = nodes[n] * dim + c;
                    u[n][c] = L->bc[dof] ? 0.0 : x[dof];
                    out[n][c] = 0.0;
                }
            for (int j = 0; j < nq; j++) {
                int pt[3] = {j % 3, (j / 3) % 3, dim == 3 ? j / 9 : 1};
                double w = L->W[(int64_t)j * L->n_el + e];
                double gN[8][3], g[3][3] = {{0}};
                for (int n = 0; n < nen; n++)
                    for (int d = 0; d < dim; d++) gN[n][d] = hi[d] * lderiv(dim, n, d, pt);
                for (int n = 0; n < nen; n++)
                    for (int c = 0; c < dim; c++)
                        for (int d = 0; d < dim; d++) g[c][d] += u[n][c] * gN[n][d];
                double S[3][3];
                for (int c = 0; c < dim; c++)
                    for (int d = 0; d < dim; d++) S[c][d] = w * (g[c][d] + g[d][c]);
                for (int n = 0; n < nen; n++)
                    for (int c = 0; c < dim; c++) {
                        double a = 0.0;
                        for (int d = 0; d < dim; d++) a += gN[n][d] * S[c][d];
                        out[n][c] += a;
                    }
            }
            for (int n = 0; n < nen; n++)
                for (int c = 0; c < dim; c++) {
                    int64_t dof = nodes[n] * dim + c;
                    if (!L->bc[dof]) y[dof] += out[n][c];
                }
        }
    }
}

void uwo_sys_applyK(const uwo_sys* s, int l, const double* x, double* y) { applyK(s, l, x, y); }

/* G p (dQ0) and G^T u, element closed form -int dN_A/dx_i */
static double gcoef(int dim, int n, int i, const double* h) {
    double ge = 1.0;
    for (int d = 0; d < dim; d++)
        if (d != i) ge *= 0.5 * h[d];
    return ge * (((n >> i) & 1) ? -1.0 : 1.0);
}

static void applyG(const uwo_sys* s, const double* p, double* y) {
    const lev_t* L = &s->L[0];
    int dim = s->dim, nen = dim == 3 ? 8 : 4;
    memset(y, 0, sizeof(double) * s->nv);
    for (int color = 0; color < (1 << dim); color++) {
#pragma omp parallel for schedule(static)
        for (int64_t e = 0; e < L->n_el; e++) {
            int ex = (int)(e % L->res[0]), ey = (int)((e / L->res[0]) % L->res[1]);
            int ez = dim == 3 ? (int)(e / ((int64_t)L->res[0] * L->res[1])) : 0;
            if (((ex & 1) | ((ey & 1) << 1) | ((ez & 1) << 2)) != color) continue;
            int64_t nodes[8];
            double h[3];
            elem(s, L, e, nodes, h);
            for (int n = 0; n < nen; n++)
                for (int i = 0; i < dim; i++) {
                    int64_t dof = nodes[n] * dim + i;
                    if (!L->bc[dof]) y[dof] += gcoef(dim, n, i, h) * p[e];
                }
        }
    }
}

static void applyGt(const uwo_sys* s, const double* u, double* q, int only_bc) {
    const lev_t* L = &s->L[0];
    int dim = s->dim, nen = dim == 3 ? 8 : 4;
#pragma omp parallel for schedule(static)
    for (int64_t e = 0; e < L->n_el; e++) {
        int64_t nodes[8];
        double h[3], a = 0.0;
        elem(s, L, e, nodes, h);
        for (int n = 0; n < nen; n++)
            for (int i = 0; i < dim; i++) {
                int64_t dof = nodes[n] * dim + i;
                if ((L->bc[dof] != 0) != (only_bc != 0)) continue;
                a += gcoef(dim, n, i, h) * u[dof];
            }
        q[e] = a;
    }
}

static double dot(int64_t n, const double* a, const double* b) {
    double s = 0.0;
#pragma omp parallel for reduction(+ : s) schedule(static)
    for (int64_t i = 0; i < n; i++) s += a[i] * b[i];
    return s;
}

static void axpy(int64_t n, double a, const double* x, double* y) {
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n; i++) y[i] += a * x[i];
}

/* element diagonal, Schur block, W coarsening, dense coarse inverse */
static void level_setup(uwo_sys* s, int l) {
    lev_t* L = &s->L[l];
    int dim = s->dim, nq = s->nq, nen = dim == 3 ? 8 : 4;
    memset(L->diag, 0, sizeof(double) * L->n_dof);
    for (int color = 0; color < (1 << dim); color++) {
#pragma omp parallel for schedule(static)
        for (int64_t e = 0; e < L->n_el; e++) {
            int ex = (int)(e % L->res[0]), ey = (int)((e / L->res[0]) % L->res[1]);
            int ez = dim == 3 ? (int)(e / ((int64_t)L->res[0] * L->res[1])) : 0;
            if (((ex & 1) | ((ey & 1) << 1) | ((ez & 1) << 2)) != color) continue;
            int64_t nodes[8];
            double h[3], kd[24] = {0};
            elem(s, L, e, nodes, h);
            double hi[3] = {2.0 / h[0], 2.0 / h[1], 2.0 / h[2]};
            for (int j = 0; j < nq; j++) {
                int pt[3] = {j % 3, (j / 3) % 3, dim == 3 ? j / 9 : 1};
                double w = L->W[(int64_t)j * L->n_el + e];
                for (int n = 0; n < nen; n++) {
                    double gx[3], s2 = 0.0;
                    for (int d = 0; d < dim; d++) { gx[d] = hi[d] * lderiv(dim, n, d, pt); s2 += gx[d] * gx[d]; }
                    for (int c = 0; c < dim; c++) kd[n * dim + c] += w * (s2 + gx[c] * gx[c]);
                }
            }
            for (int n = 0; n < nen; n++)
                for (int c = 0; c < dim; c++) {
                    int64_t dof = nodes[n] * dim + c;
                    if (!L->bc[dof]) L->diag[dof] += kd[n * dim + c];
                }
            if (l == 0) {
                double sh = 0.0;
                for (int n = 0; n < nen; n++)
                    for (int i = 0; i < dim; i++) {
                        double ge = gcoef(dim, n, i, h);
                        sh += ge * (ge / kd[n * dim + i]);
                    }
                s->shat[e] = sh;
            }
        }
    }
    for (int64_t i = 0; i < L->n_dof; i++)
        if (L->bc[i]) L->diag[i] = 1.0;
}

static void coarsen(uwo_sys* s, int l) {
    lev_t *F = &s->L[l], *C = &s->L[l + 1];
    int dim = s->dim, nq = s->nq;
    double T[2][3][3];
    for (int dl = 0; dl < 2; dl++)
        for (int b = 0; b < 3; b++) {
            double x = ((b - 1) + (2 * dl - 1)) * 0.5;
            T[dl][b][0] = 0.5 * x * (x - 1.0); T[dl][b][1] = 1.0 - x * x; T[dl][b][2] = 0.5 * x * (x + 1.0);
        }
#pragma omp parallel for schedule(static)
    for (int64_t e = 0; e < C->n_el; e++) {
        int ex = (int)(e % C->res[0]), ey = (int)((e / C->res[0]) % C->res[1]);
        int ez = dim == 3 ? (int)(e / ((int64_t)C->res[0] * C->res[1])) : 0;
        double acc[27] = {0};
        for (int cz = 0; cz < (dim == 3 ? 2 : 1); cz++)
            for (int cy = 0; cy < 2; cy++)
                for (int cx = 0; cx < 2; cx++) {
                    int64_t fe = (2 * ex + cx) + (int64_t)F->res[0] * ((2 * ey + cy) + (int64_t)F->res[1] * (2 * ez + cz));
                    for (int j = 0; j < nq; j++) {
                        double w = F->W[(int64_t)j * F->n_el + fe];
                        int jx = j % 3, jy = (j / 3) % 3, jz = j / 9;
                        for (int a = 0; a < nq; a++) {
                            int ax = a % 3, ay = (a / 3) % 3, az = a / 9;
                            double t = T[cx][jx][ax] * T[cy][jy][ay] * (dim == 3 ? T[cz][jz][az] : 1.0);
                            acc[a] += w * t;
                        }
                    }
                }
        for (int j = 0; j < nq; j++) C->W[(int64_t)j * C->n_el + e] = acc[j];
    }
}

static void dense_coarse(uwo_sys* s, int l) {
    lev_t* L = &s->L[l];
    int dim = s->dim, nen = dim == 3 ? 8 : 4;
    int64_t n = L->n_dof;
    double* A = dalloc(n * n);
    double* e_ = dalloc(n);
    double* y = dalloc(n);
    for (int64_t j = 0; j < n; j++) {           /* columns by unit applies (n is tiny) */
        memset(e_, 0, sizeof(double) * n);
        e_[j] = 1.0;
        applyK(s, l, e_, y);
        for (int64_t i = 0; i < n; i++) A[i * n + j] = y[i];
    }
    (void)nen;
    double* B = L->cinv;
    for (int64_t i = 0; i < n * n; i++) B[i] = (i / n == i % n) ? 1.0 : 0.0;
    for (int64_t k = 0; k < n; k++) {
        double piv = A[k * n + k];
        for (int64_t j = 0; j < n; j++) { A[k * n + j] /= piv; B[k * n + j] /= piv; }
        for (int64_t i = 0; i < n; i++) {
            if (i == k) continue;
            double f = A[i * n + k];
            if (f == 0.0) continue;
            for (int64_t j = 0; j < n; j++) { A[i * n + j] -= f * A[k * n + j]; B[i * n + j] -= f * B[k * n + j]; }
        }
    }
    free(A); free(e_); free(y);
}

static void estimate(uwo_sys* s, int l) {
    lev_t* L = &s->L[l];
    int64_t n = L->n_dof;
    for (int64_t i = 0; i < n; i++) L->x[i] = L->bc[i] ? 0.0 : 1.0 + 0.37 * sin(0.731 * (double)i);
    double lam = 1.0;
    for (int it = 0; it < 12; it++) {
        applyK(s, l, L->x, L->t);
        for (int64_t i = 0; i < n; i++) L->d[i] = L->bc[i] ? 0.0 : L->t[i] / L->diag[i];
        double a = dot(n, L->d, L->d), b = dot(n, L->x, L->x);
        if (b <= 0.0) break;
        lam = sqrt(a / b);
        double sc = 1.0 / sqrt(a);
        for (int64_t i = 0; i < n; i++) L->x[i] = L->d[i] * sc;
    }
    L->lmax = lam;
}

void uwo_sys_set_bc(uwo_sys* s, const uint8_t* mask, const double* values) {
    memcpy(s->L[0].bc, mask, (size_t)s->nv);
    for (int64_t i = 0; i < s->nv; i++) s->bcval[i] = (mask[i] && values) ? values[i] : 0.0;
    for (int l = 0; l + 1 < s->nlev; l++) {
        lev_t *F = &s->L[l], *C = &s->L[l + 1];
        int64_t cnx = C->res[0] + 1, cny = C->res[1] + 1, fnx = F->res[0] + 1, fny = F->res[1] + 1;
        for (int64_t nd = 0; nd < C->n_nodes; nd++) {
            int64_t ci = nd % cnx, cj = (nd / cnx) % cny, ck = nd / (cnx * cny);
            int64_t fn = 2 * ci + fnx * (2 * cj + fny * 2 * ck);
            for (int c = 0; c < s->dim; c++) C->bc[nd * s->dim + c] = F->bc[fn * s->dim + c];
        }
    }
}

/* after uwo_sys_assemble_points: lifting, hierarchy, smoother bounds */
void uwo_sys_finish(uwo_sys* s) {
    memset(s->h, 0, sizeof(double) * s->np);
    int any = 0;
    for (int64_t i = 0; i < s->nv; i++) any |= s->bcval[i] != 0.0;
    if (any) {
        /* f -= K_fb g ; h -= G_b^T g */
        lev_t* L = &s->L[0];
        uint8_t* save = L->bc;
        uint8_t* none = (uint8_t*)calloc((size_t)s->nv, 1);
        L->bc = none;
        applyK(s, 0, s->bcval, s->u1);
        L->bc = save;
        for (int64_t i = 0; i < s->nv; i++) s->f[i] = L->bc[i] ? 0.0 : s->f[i] - s->u1[i];
        free(none);
        applyGt(s, s->bcval, s->pt1, 1);
        for (int64_t e = 0; e < s->np; e++) s->h[e] -= s->pt1[e];
    } else {
        for (int64_t i = 0; i < s->nv; i++) if (s->L[0].bc[i]) s->f[i] = 0.0;
    }
    for (int l = 0; l < s->nlev; l++) {
        if (l > 0) coarsen(s, l - 1);
        level_setup(s, l);
        if (l < s->nlev - 1) estimate(s, l);
    }
    dense_coarse(s, s->nlev - 1);
}

static void prolong_add(const uwo_sys* s, int lc, const double* xc, double* xf) {
    const lev_t *F = &s->L[lc - 1], *C = &s->L[lc];
    int dim = s->dim;
    int64_t fnx = F->res[0] + 1, fny = F->res[1] + 1, cnx = C->res[0] + 1, cny = C->res[1] + 1;
#pragma omp parallel for schedule(static)
    for (int64_t n = 0; n < F->n_nodes; n++) {
        int fi[3] = {(int)(n % fnx), (int)((n / fnx) % fny), dim == 3 ? (int)(n / (fnx * fny)) : 0};
        int lo[3], hi[3];
        double wl[3], wh[3];
        for (int d = 0; d < 3; d++) {
            if (d >= dim) { lo[d] = hi[d] = 0; wl[d] = 1; wh[d] = 0; continue; }
            if (fi[d] & 1) { lo[d] = fi[d] >> 1; hi[d] = lo[d] + 1; wl[d] = wh[d] = 0.5; }
            else { lo[d] = hi[d] = fi[d] >> 1; wl[d] = 1; wh[d] = 0; }
        }
        double acc[3] = {0, 0, 0};
        for (int kz = 0; kz < (dim == 3 ? 2 : 1); kz++)
            for (int ky = 0; ky < 2; ky++)
                for (int kx = 0; kx < 2; kx++) {
                    double w = (kx ? wh[0] : wl[0]) * (ky ? wh[1] : wl[1]) * (dim == 3 ? (kz ? wh[2] : wl[2]) : 1.0);
                    if (w == 0.0) continue;
                    int64_t cn = (kx ? hi[0] : lo[0]) + cnx * ((ky ? hi[1] : lo[1]) + cny * (int64_t)(kz ? hi[2] : lo[2]));
                    for (int c = 0; c < dim; c++) acc[c] += w * xc[cn * dim + c];
                }
        for (int c = 0; c < dim; c++)
            if (!F->bc[n * dim + c]) xf[n * dim + c] += acc[c];
    }
}

static void restrict_(const uwo_sys* s, int lc, const double* rf, double* rc) {
    const lev_t *F = &s->L[lc - 1], *C = &s->L[lc];
    int dim = s->dim;
    int64_t fnx = F->res[0] + 1, fny = F->res[1] + 1, cnx = C->res[0] + 1, cny = C->res[1] + 1;
    int64_t fnz = dim == 3 ? F->res[2] + 1 : 1;
#pragma omp parallel for schedule(static)
    for (int64_t n = 0; n < C->n_nodes; n++) {
        int ci[3] = {(int)(n % cnx), (int)((n / cnx) % cny), dim == 3 ? (int)(n / (cnx * cny)) : 0};
        double acc[3] = {0, 0, 0};
        for (int dz = (dim == 3 ? -1 : 0); dz <= (dim == 3 ? 1 : 0); dz++)
            for (int dy = -1; dy <= 1; dy++)
                for (int dx = -1; dx <= 1; dx++) {
                    int64_t f0 = 2 * ci[0] + dx, f1 = 2 * ci[1] + dy, f2 = 2 * ci[2] + dz;
                    if (f0 < 0 || f0 >= fnx || f1 < 0 || f1 >= fny || f2 < 0 || f2 >= fnz) continue;
                    double w = (dx ? 0.5 : 1.0) * (dy ? 0.5 : 1.0) * (dz ? 0.5 : 1.0);
                    int64_t fn = f0 + fnx * (f1 + fny * f2);
                    for (int c = 0; c < dim; c++)
                        if (!F->bc[fn * dim + c]) acc[c] += w * rf[fn * dim + c];
                }
        for (int c = 0; c < dim; c++) rc[n * dim + c] = C->bc[n * dim + c] ? 0.0 : acc[c];
    }
}

static void chebyshev(uwo_sys* s, int l, const double* b, double* x, int deg, int x_zero) {
    lev_t* L = &s->L[l];
    int64_t n = L->n_dof;
    double alpha = 0.1 * L->lmax, beta = 1.1 * L->lmax;
    double theta = 0.5 * (beta + alpha), delta = 0.5 * (beta - alpha);
    double sigma = theta / delta, rho = 1.0 / sigma;
    if (x_zero) memcpy(L->r, b, sizeof(double) * n);
    else {
        applyK(s, l, x, L->t);
#pragma omp parallel for schedule(static)
        for (int64_t i = 0; i < n; i++) L->r[i] = b[i] - L->t[i];
    }
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n; i++) { L->d[i] = L->r[i] / L->diag[i] / theta; x[i] += L->d[i]; }
    for (int k = 1; k < deg; k++) {
        applyK(s, l, x, L->t);
        double rho1 = 1.0 / (2.0 * sigma - rho);
        double a = 2.0 * rho1 / delta, c = rho1 * rho;
#pragma omp parallel for schedule(static)
        for (int64_t i = 0; i < n; i++) {
            double r = b[i] - L->t[i];
            L->d[i] = a * (r / L->diag[i]) + c * L->d[i];
            x[i] += L->d[i];
        }
        rho = rho1;
    }
}

static void vcycle(uwo_sys* s, int l, const double* b, double* x, int deg) {
    lev_t* L = &s->L[l];
    int64_t n = L->n_dof;
    if (l == s->nlev - 1) {
#pragma omp parallel for schedule(static)
        for (int64_t i = 0; i < n; i++) {
            double a = 0.0;
            for (int64_t j = 0; j < n; j++) a += L->cinv[i * n + j] * b[j];
            x[i] = a;
        }
        return;
    }
    lev_t* C = &s->L[l + 1];
    memset(x, 0, sizeof(double) * n);
    chebyshev(s, l, b, x, deg, 1);
    applyK(s, l, x, L->t);
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n; i++) L->t[i] = b[i] - L->t[i];
    restrict_(s, l + 1, L->t, C->b);
    vcycle(s, l + 1, C->b, C->x, deg);
    prolong_add(s, l + 1, C->x, x);
    chebyshev(s, l, b, x, deg, 0);
}

/* MG-preconditioned CG, x from zero; returns iterations (negative: cap hit) */
static int pcg(uwo_sys* s, const double* b, double* x, double tol, int maxit, int deg) {
    int64_t n = s->nv;
    double bn = sqrt(dot(n, b, b));
    memset(x, 0, sizeof(double) * n);
    if (bn == 0.0) return 0;
    double *r = s->cg_r, *z = s->cg_z, *p = s->cg_p, *q = s->cg_q;
    memcpy(r, b, sizeof(double) * n);
    vcycle(s, 0, r, z, deg);
    memcpy(p, z, sizeof(double) * n);
    double rz = dot(n, r, z);
    for (int it = 1; it <= maxit; it++) {
        applyK(s, 0, p, q);
        double alpha = rz / dot(n, p, q);
        axpy(n, alpha, p, x);
        axpy(n, -alpha, q, r);
        if (sqrt(dot(n, r, r)) <= tol * bn) return it;
        vcycle(s, 0, r, z, deg);
        double rz1 = dot(n, r, z), beta = rz1 / rz;
        rz = rz1;
#pragma omp parallel for schedule(static)
        for (int64_t i = 0; i < n; i++) p[i] = z[i] + beta * p[i];
    }
    return -maxit;
}

static int schur(uwo_sys* s, const double* p, double* q, double tol, int maxit, int deg) {
    applyG(s, p, s->u1);
    int it = pcg(s, s->u1, s->u2, tol, maxit, deg);
    applyGt(s, s->u2, q, 0);
#pragma omp parallel for schedule(static)
    for (int64_t e = 0; e < s->np; e++) q[e] = -q[e];
    return it < 0 ? -it : it;
}

/* stats: [0] pressure its, [1] presolve its, [2] pressure-solve velocity its,
 * [3] backsolve its, [4] relative residual.  Returns 0 or -1 (cap hit). */
int uwo_sys_solve(uwo_sys* s, double inner_rtol, double outer_rtol, int max_inner, int max_outer, int deg,
                  double* u, double* p, double* stats) {
    int64_t nv = s->nv, np = s->np;
    int m = s->restart, rc = 0;
    for (int64_t i = 0; i < nv; i++) s->bvec[i] = s->L[0].bc[i] ? s->bcval[i] : s->f[i];
    int it_pre = pcg(s, s->bvec, s->ftil, inner_rtol, max_inner, deg);
    if (it_pre < 0) { rc = -1; it_pre = -it_pre; }
    for (int64_t i = 0; i < nv; i++) if (s->L[0].bc[i]) s->ftil[i] = 0.0;
    applyGt(s, s->ftil, s->hhat, 0);
    for (int64_t e = 0; e < np; e++) s->hhat[e] = s->h[e] - s->hhat[e];
    /* FGMRES(m), right preconditioner -S^-1 */
    double bn = sqrt(dot(np, s->hhat, s->hhat));
    /* stop once the Schur residual is below half the full-system target (1e-8) */
    double fnorm = 0.0;
    for (int64_t i = 0; i < nv; i++) if (!s->L[0].bc[i]) fnorm += s->f[i] * s->f[i];
    for (int64_t e = 0; e < np; e++) fnorm += s->h[e] * s->h[e];
    double tol = outer_rtol * bn, atol = 0.5e-8 * sqrt(fnorm);
    if (atol > 0.0 && atol < tol) tol = atol;
    memset(p, 0, sizeof(double) * np);
    int total = 0, inner_its = 0;
    double* H = (double*)calloc((size_t)(m + 1) * m, sizeof(double));
    double *cs = dalloc(m), *sn = dalloc(m), *g = dalloc(m + 1), *y = dalloc(m);
    if (bn > 0.0) {
        memcpy(s->V[0], s->hhat, sizeof(double) * np);
        double beta = bn;
        int done = 0;
        while (!done && total < max_outer) {
            for (int64_t e = 0; e < np; e++) s->V[0][e] /= beta;
            memset(g, 0, sizeof(double) * (m + 1));
            g[0] = beta;
            int j = 0;
            for (; j < m && total < max_outer; j++) {
                for (int64_t e = 0; e < np; e++) s->Z[j][e] = -s->V[j][e] / s->shat[e];
                inner_its += schur(s, s->Z[j], s->V[j + 1], inner_rtol, max_inner, deg);
                total++;
                for (int pass = 0; pass < 2; pass++)
                    for (int i = 0; i <= j; i++) {
                        double hij = dot(np, s->V[i], s->V[j + 1]);
                        H[i * m + j] += hij;
                        axpy(np, -hij, s->V[i], s->V[j + 1]);
                    }
                double hn = sqrt(dot(np, s->V[j + 1], s->V[j + 1]));
                H[(j + 1) * m + j] = hn;
                for (int i = 0; i < j; i++) {
                    double t = cs[i] * H[i * m + j] + sn[i] * H[(i + 1) * m + j];
                    H[(i + 1) * m + j] = -sn[i] * H[i * m + j] + cs[i] * H[(i + 1) * m + j];
                    H[i * m + j] = t;
                }
                double a = H[j * m + j], b = H[(j + 1) * m + j], r = hypot(a, b);
                cs[j] = r == 0.0 ? 1.0 : a / r;
                sn[j] = r == 0.0 ? 0.0 : b / r;
                H[j * m + j] = r;
                H[(j + 1) * m + j] = 0.0;
                g[j + 1] = -sn[j] * g[j];
                g[j] = cs[j] * g[j];
                if (hn > 0.0) for (int64_t e = 0; e < np; e++) s->V[j + 1][e] /= hn;
                if (fabs(g[j + 1]) <= tol || hn == 0.0) { j++; done = 1; break; }
            }
            for (int i = j - 1; i >= 0; i--) {
                double t = g[i];
                for (int k = i + 1; k < j; k++) t -= H[i * m + k] * y[k];
                y[i] = t / H[i * m + i];
            }
            for (int i = 0; i < j; i++) axpy(np, y[i], s->Z[i], p);
            memset(H, 0, sizeof(double) * (size_t)(m + 1) * m);
            if (!done) {
                inner_its += schur(s, p, s->pt1, inner_rtol, max_inner, deg);
                for (int64_t e = 0; e < np; e++) s->V[0][e] = s->hhat[e] - s->pt1[e];
                beta = sqrt(dot(np, s->V[0], s->V[0]));
                if (beta <= tol) done = 1;
            }
        }
        if (!done) rc = -1;
    }
    free(H); free(cs); free(sn); free(g); free(y);
    /* back-solve */
    applyG(s, p, s->u1);
    for (int64_t i = 0; i < nv; i++) s->u1[i] = s->bvec[i] - s->u1[i];
    int it_back = pcg(s, s->u1, u, inner_rtol, max_inner, deg);
    if (it_back < 0) { rc = -1; it_back = -it_back; }
    /* residual of the full system over free dofs */
    applyK(s, 0, u, s->u1);
    applyG(s, p, s->u2);
    double rn = 0.0, fn = 0.0;
    for (int64_t i = 0; i < nv; i++) {
        if (s->L[0].bc[i]) continue;
        double r = s->f[i] - s->u1[i] - s->u2[i];
        rn += r * r;
        fn += s->f[i] * s->f[i];
    }
    applyGt(s, u, s->pt1, 0);
    for (int64_t e = 0; e < np; e++) {
        double r = s->h[e] - s->pt1[e];
        rn += r * r;
        fn += s->h[e] * s->h[e];
    }
    stats[0] = total; stats[1] = it_pre; stats[2] = inner_its; stats[3] = it_back;
    stats[4] = fn > 0.0 ? sqrt(rn / fn) : sqrt(rn);
    return rc;
}
