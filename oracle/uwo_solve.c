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
#include <time.h>
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
    /* Schur preconditioner: 0 the assembled Uzawa term, 1 weighted scaled BFBt */
    int schur_pc, pc_deg;
    double pc_rtol;
    struct pmg_s* pmg;
} uwo_sys;

struct pmg_s;
static void pmg_free(struct pmg_s* P);
static struct pmg_s* pmg_setup(const uwo_sys* s, int deg);

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
    pmg_free(s->pmg);
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
    pmg_free(s->pmg);
    s->pmg = s->schur_pc == 1 ? pmg_setup(s, s->pc_deg) : NULL;
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

/* ------------------------------------------------------------------------ */
/* Weighted scaled BFBt Schur preconditioner, the GPU library's default      */
/* (May & Moresi 2008; square-root diagonal weight, Rudi et al. 2017):      */
/*   S^-1 ~ -L^-1 (G^T W K W G) L^-1,  L = G^T W G,  W = diag(K)^-1/2,      */
/* with L^-1 by multigrid-preconditioned CG to a relative 3e-2.  The        */
/* pressure multigrid carries a smooth and a checkerboard unknown per       */
/* coarse cell; level 1 interpolates the checkerboard part cell-centred     */
/* trilinearly (when there are >= 3 levels), deeper levels aggregate        */
/* piecewise constantly; coarse operators are Galerkin products.  FP32      */
/* storage as on the GPU, so both arms run the same algorithm and move      */
/* the same bytes per iteration.                                            */
/* ------------------------------------------------------------------------ */
typedef struct pmg_s {
    int on, smooth1, deg, nlev, dim, no, n5;
    int64_t n[MAXLEV];
    int res[MAXLEV][3];
    float* st[MAXLEV];    /* level 0: [no][n]; level >= 1: [no][2][2][n] (+ level-1 cc5 [n5][n]) */
    float* cc5;
    float* dg[MAXLEV];    /* [nc][n] */
    double lmax[MAXLEV];
    float *r[MAXLEV], *x[MAXLEV], *b[MAXLEV], *t[MAXLEV], *d[MAXLEV];
    float* cinv;          /* dense inverse of the coarsest level */
    int64_t mc;
    double* w0;           /* 1/sqrt(diag K) on free velocity dofs, 0 on Dirichlet dofs */
    float *cr, *cz, *cp, *cq, *cx, *fr, *fz, *f1, *f2;
    double *v1, *v2;
    int its;              /* L-solve CG iterations (statistics) */
} pmg_t;

static int pmg_nc(int l) { return l == 0 ? 1 : 2; }
static float* fal(int64_t n) { return (float*)calloc((size_t)(n > 0 ? n : 1), sizeof(float)); }

static void pcell(const pmg_t* P, int l, int64_t e, int* X) {
    X[0] = (int)(e % P->res[l][0]);
    X[1] = (int)((e / P->res[l][0]) % P->res[l][1]);
    X[2] = P->dim == 3 ? (int)(e / ((int64_t)P->res[l][0] * P->res[l][1])) : 0;
}
static int pin(const pmg_t* P, int l, int x, int y, int z) {
    return x >= 0 && x < P->res[l][0] && y >= 0 && y < P->res[l][1] && (P->dim == 2 || (z >= 0 && z < P->res[l][2]));
}
static int64_t pidx(const pmg_t* P, int l, int x, int y, int z) {
    return x + (int64_t)P->res[l][0] * (y + (int64_t)P->res[l][1] * z);
}
static int coff(int c, int o) { return ((c + o + 2) >> 1) - 1; }

/* |int dN/dx_d| over cell (x,y,z) of level 0 per axis (face areas / 4 in 3D) */
static void gco(const uwo_sys* s, int ex, int ey, int ez, float* a) {
    const lev_t* L = &s->L[0];
    float hx = (float)(L->ax[0][ex + 1] - L->ax[0][ex]), hy = (float)(L->ax[1][ey + 1] - L->ax[1][ey]);
    float hz = s->dim == 3 ? (float)(L->ax[2][ez + 1] - L->ax[2][ez]) : 2.0f;
    a[0] = 0.5f * hy * (s->dim == 3 ? 0.5f * hz : 1.0f);
    a[1] = 0.5f * hx * (s->dim == 3 ? 0.5f * hz : 1.0f);
    a[2] = 0.25f * hx * hy;
}

/* level-0 stencil of L = G^T W G (W zero on Dirichlet dofs) */
static void pst0(const uwo_sys* s, pmg_t* P) {
    int dim = s->dim, no = P->no;
    const lev_t* L = &s->L[0];
    int64_t n = P->n[0], nx = L->res[0] + 1, ny = L->res[1] + 1;
    float* st = P->st[0];
#pragma omp parallel for schedule(static)
    for (int64_t e = 0; e < n; e++) {
        int X[3];
        pcell(P, 0, e, X);
        float a[3], acc[27];
        gco(s, X[0], X[1], X[2], a);
        for (int o = 0; o < no; o++) acc[o] = 0.f;
        for (int ln = 0; ln < (1 << dim); ln++) {
            int lx = ln & 1, ly = (ln >> 1) & 1, lz = dim == 3 ? (ln >> 2) & 1 : 0;
            int64_t node = (X[0] + lx) + nx * ((X[1] + ly) + ny * (int64_t)(X[2] + lz));
            float w[3] = {0.f, 0.f, 0.f};
            for (int d = 0; d < dim; d++) w[d] = (float)P->w0[node * dim + d];
            float ge0 = lx ? -a[0] : a[0], ge1 = ly ? -a[1] : a[1], ge2 = lz ? -a[2] : a[2];
            for (int cn = 0; cn < (1 << dim); cn++) {
                int cx = cn & 1, cy = (cn >> 1) & 1, cz = dim == 3 ? (cn >> 2) & 1 : 0;
                int fx = X[0] + lx - 1 + cx, fy = X[1] + ly - 1 + cy, fz = dim == 3 ? X[2] + lz - 1 + cz : 0;
                if (!pin(P, 0, fx, fy, fz)) continue;
                float b[3];
                gco(s, fx, fy, fz, b);
                float v = w[0] * ge0 * (cx ? b[0] : -b[0]) + w[1] * ge1 * (cy ? b[1] : -b[1]);
                if (dim == 3) v += w[2] * ge2 * (cz ? b[2] : -b[2]);
                acc[(lx + cx) + 3 * (ly + cy) + (dim == 3 ? 9 * (lz + cz) : 0)] += v;
            }
        }
        for (int o = 0; o < no; o++) st[o * n + e] = acc[o];
    }
}

/* Galerkin level 0 -> 1, piecewise checkerboard interpolation */
static void pgal01(pmg_t* P) {
    int dim = P->dim, no = P->no;
    int64_t nf = P->n[0], nc = P->n[1];
#pragma omp parallel for schedule(static)
    for (int64_t I = 0; I < nc; I++) {
        int X[3];
        pcell(P, 1, I, X);
        float acc[27][4];
        memset(acc, 0, sizeof(acc));
        for (int cn = 0; cn < (1 << dim); cn++) {
            int cx = cn & 1, cy = (cn >> 1) & 1, cz = dim == 3 ? (cn >> 2) & 1 : 0;
            int64_t i = pidx(P, 0, 2 * X[0] + cx, 2 * X[1] + cy, 2 * X[2] + cz);
            float si = ((cx + cy + cz) & 1) ? -1.f : 1.f;
            for (int o = 0; o < no; o++) {
                int ox = o % 3 - 1, oy = (o / 3) % 3 - 1, oz = dim == 3 ? o / 9 - 1 : 0;
                float v = P->st[0][o * nf + i];
                float sj = ((cx + ox + cy + oy + cz + oz) & 1) ? -1.f : 1.f;
                int O = (coff(cx, ox) + 1) + 3 * (coff(cy, oy) + 1) + (dim == 3 ? 9 * (coff(cz, oz) + 1) : 0);
                acc[O][0] += v; acc[O][1] += sj * v; acc[O][2] += si * v; acc[O][3] += si * sj * v;
            }
        }
        for (int o = 0; o < no; o++)
            for (int k = 0; k < 4; k++) P->st[1][(o * 4 + k) * nc + I] = acc[o][k];
    }
}

/* 1D trilinear support of fine cell f: (p, 3/4) and (q, 1/4), q clipped to p at the walls */
static void tri1d(int f, int rc, int* p, int* q) {
    *p = f >> 1;
    *q = (f & 1) ? *p + 1 : *p - 1;
    if (*q < 0 || *q >= rc) *q = *p;
}
static float tri1w(int f, int rc, int I) {
    int p, q;
    tri1d(f, rc, &p, &q);
    return (p == I ? 0.75f : 0.f) + (q == I ? 0.25f : 0.f);
}

/* Galerkin level 0 -> 1 with the smooth checkerboard interpolation */
static void pgal01_tri(pmg_t* P) {
    int dim = P->dim, no = P->no, n5 = P->n5, nfc = dim == 3 ? 64 : 16;
    int64_t nf = P->n[0], nc = P->n[1];
    const int* rc = P->res[1];
#pragma omp parallel for schedule(dynamic, 64)
    for (int64_t I = 0; I < nc; I++) {
        int X[3];
        pcell(P, 1, I, X);
        float ss[27], sc[27], cs[27], cc[125];
        memset(ss, 0, sizeof(ss)); memset(sc, 0, sizeof(sc)); memset(cs, 0, sizeof(cs)); memset(cc, 0, sizeof(cc));
        /* rows of the smooth component: the children of I */
        for (int ch = 0; ch < (1 << dim); ch++)
            for (int o = 0; o < no; o++) {
                int ix = 2 * X[0] + (ch & 1), iy = 2 * X[1] + ((ch >> 1) & 1), iz = dim == 3 ? 2 * X[2] + (ch >> 2) : 0;
                float v = P->st[0][o * nf + pidx(P, 0, ix, iy, iz)];
                if (v == 0.f) continue;
                int jx = ix + o % 3 - 1, jy = iy + (o / 3) % 3 - 1, jz = dim == 3 ? iz + o / 9 - 1 : 0;
                if (!pin(P, 0, jx, jy, jz)) continue;
                ss[((jx >> 1) - X[0] + 1) + 3 * ((jy >> 1) - X[1] + 1) + (dim == 3 ? 9 * ((jz >> 1) - X[2] + 1) : 0)] += v;
                float vj = ((jx + jy + jz) & 1) ? -v : v;
                int px, qx, py, qy, pz = 0, qz = 0;
                tri1d(jx, rc[0], &px, &qx);
                tri1d(jy, rc[1], &py, &qy);
                if (dim == 3) tri1d(jz, rc[2], &pz, &qz);
                for (int cz = 0; cz < (dim == 3 ? 2 : 1); cz++)
                    for (int cy = 0; cy < 2; cy++)
                        for (int cx = 0; cx < 2; cx++) {
                            int Jx = cx ? qx : px, Jy = cy ? qy : py, Jz = cz ? qz : pz;
                            float w = (cx ? 0.25f : 0.75f) * (cy ? 0.25f : 0.75f) * (dim == 3 ? (cz ? 0.25f : 0.75f) : 1.f);
                            sc[(Jx - X[0] + 1) + 3 * (Jy - X[1] + 1) + (dim == 3 ? 9 * (Jz - X[2] + 1) : 0)] += w * vj;
                        }
            }
        /* rows of the checkerboard component: the fine cells of I's trilinear support */
        for (int f = 0; f < nfc; f++)
            for (int o = 0; o < no; o++) {
                int ix = 2 * X[0] - 1 + (f & 3), iy = 2 * X[1] - 1 + ((f >> 2) & 3), iz = dim == 3 ? 2 * X[2] - 1 + (f >> 4) : 0;
                if (!pin(P, 0, ix, iy, iz)) continue;
                float wi = tri1w(ix, rc[0], X[0]) * tri1w(iy, rc[1], X[1]) * (dim == 3 ? tri1w(iz, rc[2], X[2]) : 1.f);
                if (wi == 0.f) continue;
                float v0 = P->st[0][o * nf + pidx(P, 0, ix, iy, iz)];
                if (v0 == 0.f) continue;
                float v = (((ix + iy + iz) & 1) ? -wi : wi) * v0;
                int jx = ix + o % 3 - 1, jy = iy + (o / 3) % 3 - 1, jz = dim == 3 ? iz + o / 9 - 1 : 0;
                if (!pin(P, 0, jx, jy, jz)) continue;
                cs[((jx >> 1) - X[0] + 1) + 3 * ((jy >> 1) - X[1] + 1) + (dim == 3 ? 9 * ((jz >> 1) - X[2] + 1) : 0)] += v;
                float vj = ((jx + jy + jz) & 1) ? -v : v;
                int px, qx, py, qy, pz = 0, qz = 0;
                tri1d(jx, rc[0], &px, &qx);
                tri1d(jy, rc[1], &py, &qy);
                if (dim == 3) tri1d(jz, rc[2], &pz, &qz);
                for (int cz = 0; cz < (dim == 3 ? 2 : 1); cz++)
                    for (int cy = 0; cy < 2; cy++)
                        for (int cx = 0; cx < 2; cx++) {
                            int Jx = cx ? qx : px, Jy = cy ? qy : py, Jz = cz ? qz : pz;
                            float w = (cx ? 0.25f : 0.75f) * (cy ? 0.25f : 0.75f) * (dim == 3 ? (cz ? 0.25f : 0.75f) : 1.f);
                            cc[(Jx - X[0] + 2) + 5 * (Jy - X[1] + 2) + (dim == 3 ? 25 * (Jz - X[2] + 2) : 0)] += w * vj;
                        }
            }
        for (int k = 0; k < n5; k++) P->cc5[k * nc + I] = cc[k];
        for (int k = 0; k < no; k++) {
            P->st[1][(k * 4 + 0) * nc + I] = ss[k];
            P->st[1][(k * 4 + 1) * nc + I] = sc[k];
            P->st[1][(k * 4 + 2) * nc + I] = cs[k];
            P->st[1][(k * 4 + 3) * nc + I] = 0.f;
        }
    }
}

/* Galerkin level l -> l+1, two unknowns per cell on both (aggregation per
 * component); from level 1 with the smooth checkerboard block when tri */
static void pgal2(pmg_t* P, int lc, int from_tri) {
    int dim = P->dim, no = P->no, n5 = P->n5;
    int64_t nf = P->n[lc - 1], nc = P->n[lc];
#pragma omp parallel for schedule(static)
    for (int64_t I = 0; I < nc; I++) {
        int X[3];
        pcell(P, lc, I, X);
        float acc[27][4];
        memset(acc, 0, sizeof(acc));
        for (int cn = 0; cn < (1 << dim); cn++) {
            int cx = cn & 1, cy = (cn >> 1) & 1, cz = dim == 3 ? (cn >> 2) & 1 : 0;
            int64_t i = pidx(P, lc - 1, 2 * X[0] + cx, 2 * X[1] + cy, 2 * X[2] + cz);
            for (int o = 0; o < no; o++) {
                int ox = o % 3 - 1, oy = (o / 3) % 3 - 1, oz = dim == 3 ? o / 9 - 1 : 0;
                int O = (coff(cx, ox) + 1) + 3 * (coff(cy, oy) + 1) + (dim == 3 ? 9 * (coff(cz, oz) + 1) : 0);
                for (int k = 0; k < (from_tri ? 3 : 4); k++) acc[O][k] += P->st[lc - 1][(o * 4 + k) * nf + i];
            }
            if (from_tri)
                for (int o = 0; o < n5; o++) {
                    int ox = o % 5 - 2, oy = (o / 5) % 5 - 2, oz = dim == 3 ? o / 25 - 2 : 0;
                    int O = (((cx + ox + 4) >> 1) - 1) + 3 * (((cy + oy + 4) >> 1) - 1) +
                            (dim == 3 ? 9 * (((cz + oz + 4) >> 1) - 1) : 0);
                    acc[O][3] += P->cc5[o * nf + i];
                }
        }
        for (int o = 0; o < no; o++)
            for (int k = 0; k < 4; k++) P->st[lc][(o * 4 + k) * nc + I] = acc[o][k];
    }
}

static void papply(const pmg_t* P, int l, const float* x, float* y);
static void prestrict(const pmg_t* P, int lc, const float* rf, float* rc);
static void pprolong(const pmg_t* P, int lc, const float* xc, float* xf);

/* y = A_l x; level 1 with the smooth checkerboard block as P^T (A_0 (P x)) */
static void papply(const pmg_t* P, int l, const float* x, float* y) {
    if (l == 1 && P->smooth1) {
        memset(P->f1, 0, sizeof(float) * P->n[0]);
        pprolong(P, 1, x, P->f1);
        papply(P, 0, P->f1, P->f2);
        prestrict(P, 1, P->f2, y);
        return;
    }
    int dim = P->dim, no = P->no, nc = pmg_nc(l);
    int64_t n = P->n[l], sy = P->res[l][0], sz = (int64_t)P->res[l][0] * P->res[l][1];
    int tri = l == 1 && P->smooth1;
#pragma omp parallel for schedule(static)
    for (int64_t e = 0; e < n; e++) {
        int X[3];
        pcell(P, l, e, X);
        float a0 = 0.f, a1 = 0.f;
        for (int o = 0; o < no; o++) {
            int ox = o % 3 - 1, oy = (o / 3) % 3 - 1, oz = dim == 3 ? o / 9 - 1 : 0;
            if (!pin(P, l, X[0] + ox, X[1] + oy, X[2] + oz)) continue;
            int64_t j = e + ox + oy * sy + oz * sz;
            if (nc == 1) {
                a0 += P->st[l][o * n + e] * x[j];
            } else {
                const float* S = P->st[l];
                a0 += S[(o * 4 + 0) * n + e] * x[j] + S[(o * 4 + 1) * n + e] * x[n + j];
                a1 += S[(o * 4 + 2) * n + e] * x[j];
                if (!tri) a1 += S[(o * 4 + 3) * n + e] * x[n + j];
            }
        }
        if (tri)
            for (int o = 0; o < P->n5; o++) {
                int ox = o % 5 - 2, oy = (o / 5) % 5 - 2, oz = dim == 3 ? o / 25 - 2 : 0;
                if (!pin(P, l, X[0] + ox, X[1] + oy, X[2] + oz)) continue;
                a1 += P->cc5[o * n + e] * x[n + e + ox + oy * sy + oz * sz];
            }
        y[e] = a0;
        if (nc == 2) y[n + e] = a1;
    }
}

static void pdiag(pmg_t* P, int l) {
    int64_t n = P->n[l];
    int center = P->dim == 3 ? 13 : 4, c5 = P->dim == 3 ? 62 : 12;
    for (int64_t e = 0; e < n; e++) {
        if (l == 0) {
            float v = P->st[0][center * n + e];
            P->dg[0][e] = v > 0.f ? v : 1.f;
        } else {
            float a = P->st[l][(center * 4) * n + e];
            float b = (l == 1 && P->smooth1) ? P->cc5[c5 * n + e] : P->st[l][(center * 4 + 3) * n + e];
            P->dg[l][e] = a > 0.f ? a : 1.f;
            P->dg[l][n + e] = b > 0.f ? b : 1.f;
        }
    }
}

/* rc = P^T rf (level lc-1 -> lc) */
static void prestrict(const pmg_t* P, int lc, const float* rf, float* rc) {
    int dim = P->dim;
    int64_t nc = P->n[lc], nf = P->n[lc - 1];
    int tri = lc == 1 && P->smooth1;
#pragma omp parallel for schedule(static)
    for (int64_t I = 0; I < nc; I++) {
        int X[3];
        pcell(P, lc, I, X);
        float s0 = 0.f, s1 = 0.f;
        if (!tri) {
            for (int cn = 0; cn < (1 << dim); cn++) {
                int cx = cn & 1, cy = (cn >> 1) & 1, cz = dim == 3 ? (cn >> 2) & 1 : 0;
                int64_t i = pidx(P, lc - 1, 2 * X[0] + cx, 2 * X[1] + cy, 2 * X[2] + cz);
                if (lc == 1) { s0 += rf[i]; s1 += ((cx + cy + cz) & 1) ? -rf[i] : rf[i]; }
                else { s0 += rf[i]; s1 += rf[nf + i]; }
            }
        } else {
            for (int c = 0; c < (dim == 3 ? 4 : 1); c++) {
                int iz = dim == 3 ? 2 * X[2] - 1 + c : 0;
                if (dim == 3 && (iz < 0 || iz >= P->res[0][2])) continue;
                float wz = dim == 3 ? tri1w(iz, P->res[1][2], X[2]) : 1.f;
                for (int b = 0; b < 4; b++) {
                    int iy = 2 * X[1] - 1 + b;
                    if (iy < 0 || iy >= P->res[0][1]) continue;
                    float wy = tri1w(iy, P->res[1][1], X[1]);
                    int child_yz = (b == 1 || b == 2) && (dim == 2 || c == 1 || c == 2);
                    for (int a = 0; a < 4; a++) {
                        int ix = 2 * X[0] - 1 + a;
                        if (ix < 0 || ix >= P->res[0][0]) continue;
                        float v = rf[pidx(P, 0, ix, iy, iz)];
                        if (child_yz && (a == 1 || a == 2)) s0 += v;
                        float wv = tri1w(ix, P->res[1][0], X[0]) * wy * wz * v;
                        s1 += ((ix + iy + iz) & 1) ? -wv : wv;
                    }
                }
            }
        }
        rc[I] = s0;
        rc[nc + I] = s1;
    }
}

/* xf += P xc */
static void pprolong(const pmg_t* P, int lc, const float* xc, float* xf) {
    int dim = P->dim;
    int64_t nc = P->n[lc], nf = P->n[lc - 1];
    int tri = lc == 1 && P->smooth1;
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < nf; i++) {
        int X[3];
        pcell(P, lc - 1, i, X);
        int64_t I = pidx(P, lc, X[0] >> 1, X[1] >> 1, X[2] >> 1);
        if (lc > 1) { xf[i] += xc[I]; xf[nf + i] += xc[nc + I]; continue; }
        float c = xc[nc + I];
        if (tri) {
            int px, qx, py, qy, pz = 0, qz = 0;
            tri1d(X[0], P->res[1][0], &px, &qx);
            tri1d(X[1], P->res[1][1], &py, &qy);
            if (dim == 3) tri1d(X[2], P->res[1][2], &pz, &qz);
            c = 0.f;
            for (int cz = 0; cz < (dim == 3 ? 2 : 1); cz++)
                for (int cy = 0; cy < 2; cy++)
                    for (int cx = 0; cx < 2; cx++) {
                        float w = (cx ? 0.25f : 0.75f) * (cy ? 0.25f : 0.75f) * (dim == 3 ? (cz ? 0.25f : 0.75f) : 1.f);
                        c += w * xc[nc + pidx(P, 1, cx ? qx : px, cy ? qy : py, cz ? qz : pz)];
                    }
        }
        xf[i] += xc[I] + (((X[0] + X[1] + X[2]) & 1) ? -c : c);
    }
}

static void pcheb(pmg_t* P, int l, const float* b, float* x, int deg, int x_zero) {
    int64_t n = pmg_nc(l) * P->n[l];
    double lmax = P->lmax[l], alpha = 0.1 * lmax, beta = 1.2 * lmax;
    double theta = 0.5 * (beta + alpha), delta = 0.5 * (beta - alpha), sigma = theta / delta, rho = 1.0 / sigma;
    float *t = P->t[l], *d = P->d[l], *dg = P->dg[l];
    if (!x_zero) papply(P, l, x, t);
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n; i++) {
        float r = b[i] - (x_zero ? 0.f : t[i]);
        d[i] = (float)(1.0 / theta) * (r / dg[i]);
        x[i] = (x_zero ? 0.f : x[i]) + d[i];
    }
    for (int k = 1; k < deg; k++) {
        papply(P, l, x, t);
        double rho1 = 1.0 / (2.0 * sigma - rho);
        float a = (float)(2.0 * rho1 / delta), c = (float)(rho1 * rho);
#pragma omp parallel for schedule(static)
        for (int64_t i = 0; i < n; i++) {
            d[i] = a * ((b[i] - t[i]) / dg[i]) + c * d[i];
            x[i] += d[i];
        }
        rho = rho1;
    }
}

static void pvcycle(pmg_t* P, int l, const float* b, float* x) {
    int64_t n = pmg_nc(l) * P->n[l];
    if (l == P->nlev - 1) {
#pragma omp parallel for schedule(static)
        for (int64_t i = 0; i < n; i++) {
            double a = 0.0;
            for (int64_t j = 0; j < n; j++) a += (double)P->cinv[i * n + j] * b[j];
            x[i] = (float)a;
        }
        return;
    }
    pcheb(P, l, b, x, P->deg, 1);
    papply(P, l, x, P->t[l]);
    for (int64_t i = 0; i < n; i++) P->t[l][i] = b[i] - P->t[l][i];
    prestrict(P, l + 1, P->t[l], P->b[l + 1]);
    pvcycle(P, l + 1, P->b[l + 1], P->x[l + 1]);
    pprolong(P, l + 1, P->x[l + 1], x);
    pcheb(P, l, b, x, P->deg, 0);
}

static double fdot(int64_t n, const float* a, const float* b) {
    double s = 0.0;
#pragma omp parallel for reduction(+ : s) schedule(static)
    for (int64_t i = 0; i < n; i++) s += (double)a[i] * b[i];
    return s;
}

/* x = L^-1 b by V-cycle-preconditioned CG from zero to rtol, checked every
 * second iteration as on the GPU */
static void plsolve(pmg_t* P, const float* b, float* x, double rtol, int maxit) {
    int64_t n = P->n[0];
    float *r = P->cr, *z = P->cz, *p = P->cp, *q = P->cq;
    memset(x, 0, sizeof(float) * n);
    memcpy(r, b, sizeof(float) * n);
    pvcycle(P, 0, r, z);
    memcpy(p, z, sizeof(float) * n);
    double rz = fdot(n, r, z), bn = sqrt(fdot(n, r, r));
    if (!(bn > 0.0)) return;
    for (int it = 0; it < maxit; it++) {
        papply(P, 0, p, q);
        double pq = fdot(n, p, q);
        if (!(pq > 0.0)) break;
        float al = (float)(rz / pq);
#pragma omp parallel for schedule(static)
        for (int64_t i = 0; i < n; i++) { x[i] += al * p[i]; r[i] -= al * q[i]; }
        pvcycle(P, 0, r, z);
        double rz1 = fdot(n, r, z), rr = fdot(n, r, r);
        P->its++;
        if ((it & 1) && !(sqrt(rr) > rtol * bn)) break;
        float be = (float)(rz1 / rz);
        rz = rz1;
#pragma omp parallel for schedule(static)
        for (int64_t i = 0; i < n; i++) p[i] = z[i] + be * p[i];
    }
}

/* Gauss-Jordan inverse of a dense SPD matrix (in place into B), OpenMP over rows */
static void dense_inv(int64_t n, double* A, double* B) {
    for (int64_t i = 0; i < n * n; i++) B[i] = (i / n == i % n) ? 1.0 : 0.0;
    for (int64_t k = 0; k < n; k++) {
        double piv = A[k * n + k];
        for (int64_t j = 0; j < n; j++) { A[k * n + j] /= piv; B[k * n + j] /= piv; }
#pragma omp parallel for schedule(static)
        for (int64_t i = 0; i < n; i++) {
            if (i == k) continue;
            double f = A[i * n + k];
            if (f == 0.0) continue;
            for (int64_t j = 0; j < n; j++) { A[i * n + j] -= f * A[k * n + j]; B[i * n + j] -= f * B[k * n + j]; }
        }
    }
}

static void pmg_free(struct pmg_s* P) {
    if (!P) return;
    for (int l = 0; l < MAXLEV; l++) {
        free(P->st[l]); free(P->dg[l]); free(P->r[l]); free(P->x[l]); free(P->b[l]); free(P->t[l]); free(P->d[l]);
    }
    free(P->cc5); free(P->cinv); free(P->w0);
    free(P->cr); free(P->cz); free(P->cp); free(P->cq); free(P->cx); free(P->fr); free(P->fz); free(P->f1); free(P->f2);
    free(P->v1); free(P->v2);
    free(P);
}

/* Build the hierarchy after the velocity levels are set up (diag of K known). */
static struct pmg_s* pmg_setup(const uwo_sys* s, int deg) {
    pmg_t* P = (pmg_t*)calloc(1, sizeof(pmg_t));
    int dim = s->dim;
    P->dim = dim; P->no = dim == 3 ? 27 : 9; P->n5 = dim == 3 ? 125 : 25; P->deg = deg;
    int pn = 1;
    while (pn < s->nlev && (pn < 2 || s->L[pn - 1].n_el > 512)) pn++;
    P->nlev = pn;
    P->smooth1 = pn >= 3;
    for (int l = 0; l < pn; l++) {
        P->n[l] = s->L[l].n_el;
        for (int d = 0; d < 3; d++) P->res[l][d] = s->L[l].res[d];
        int64_t m = pmg_nc(l) * P->n[l];
        P->st[l] = fal((int64_t)P->no * (l == 0 ? 1 : 4) * P->n[l]);
        P->dg[l] = fal(m); P->r[l] = fal(m); P->x[l] = fal(m); P->b[l] = fal(m); P->t[l] = fal(m); P->d[l] = fal(m);
    }
    if (P->smooth1) P->cc5 = fal((int64_t)P->n5 * P->n[1]);
    int64_t n0 = P->n[0];
    P->cr = fal(n0); P->cz = fal(n0); P->cp = fal(n0); P->cq = fal(n0); P->cx = fal(n0); P->fr = fal(n0); P->fz = fal(n0);
    P->f1 = fal(n0); P->f2 = fal(n0);
    P->v1 = dalloc(s->nv); P->v2 = dalloc(s->nv);
    P->w0 = dalloc(s->nv);
    for (int64_t i = 0; i < s->nv; i++) P->w0[i] = s->L[0].bc[i] ? 0.0 : (double)(float)(1.0 / sqrt(s->L[0].diag[i]));
    pst0(s, P);
    for (int l = 1; l < pn; l++) {
        if (l == 1 && P->smooth1) pgal01_tri(P);
        else if (l == 1) pgal01(P);
        else pgal2(P, l, l == 2 && P->smooth1);
    }
    for (int l = 0; l < pn; l++) pdiag(P, l);
    /* Chebyshev bounds: power iteration on D^-1 A, as the GPU library */
    for (int l = 0; l + 1 < pn; l++) {
        int64_t m = pmg_nc(l) * P->n[l];
        float *x = P->x[l], *t = P->t[l], *d = P->d[l];
        for (int64_t i = 0; i < m; i++) x[i] = (float)(1.0 + 0.41 * sin(1.37 * (double)i) + ((i & 1) ? 0.3 : -0.3));
        double lam = 1.0;
        for (int it = 0; it < 30; it++) {
            papply(P, l, x, t);
            for (int64_t i = 0; i < m; i++) d[i] = t[i] / P->dg[l][i];
            double dd = fdot(m, d, d), xx = fdot(m, x, x);
            if (dd <= 0.0 || xx <= 0.0) break;
            lam = sqrt(dd / xx);
            float sc = (float)(1.0 / sqrt(dd));
            for (int64_t i = 0; i < m; i++) x[i] = d[i] * sc;
        }
        P->lmax[l] = lam;
    }
    /* dense inverse of the coarsest level, with tau 1 1^T on its smooth block */
    {
        int l = pn - 1, nc = pmg_nc(l), dimv = dim;
        int64_t n = P->n[l], m = nc * n;
        double* A = (double*)calloc((size_t)(m * m), sizeof(double));
        double* B = (double*)calloc((size_t)(m * m), sizeof(double));
        for (int64_t e = 0; e < n; e++) {
            int X[3];
            pcell(P, l, e, X);
            for (int o = 0; o < P->no; o++) {
                int ox = o % 3 - 1, oy = (o / 3) % 3 - 1, oz = dimv == 3 ? o / 9 - 1 : 0;
                if (!pin(P, l, X[0] + ox, X[1] + oy, X[2] + oz)) continue;
                int64_t j = e + ox + (int64_t)oy * P->res[l][0] + (int64_t)oz * P->res[l][0] * P->res[l][1];
                for (int a = 0; a < nc; a++)
                    for (int b = 0; b < nc; b++)
                        A[(a * n + e) * m + b * n + j] = P->st[l][(nc == 1 ? o : o * 4 + a * 2 + b) * n + e];
            }
        }
        double mx = 0.0;
        for (int64_t i = 0; i < n; i++) mx = fmax(mx, A[i * m + i]);
        double tau = (mx > 0.0 ? mx : 1.0) / (double)n;
        for (int64_t i = 0; i < n; i++)
            for (int64_t j = 0; j < n; j++) A[i * m + j] += tau;
        dense_inv(m, A, B);
        P->cinv = fal(m * m);
        for (int64_t i = 0; i < m * m; i++) P->cinv[i] = (float)B[i];
        P->mc = m;
        free(A); free(B);
    }
    P->on = 1;
    return P;
}

/* z = -BFBt(r) with the constant (a null mode of S) projected out of z */
static void bfbt_apply(uwo_sys* s, pmg_t* P, const double* r, double* z, double rtol) {
    int64_t np = s->np, nv = s->nv;
    for (int64_t e = 0; e < np; e++) P->fr[e] = (float)r[e];
    plsolve(P, P->fr, P->fz, rtol, 200);
    for (int64_t e = 0; e < np; e++) s->pt2[e] = P->fz[e];
    applyG(s, s->pt2, P->v1);
    for (int64_t i = 0; i < nv; i++) P->v1[i] = (double)(float)(P->v1[i] * P->w0[i]);
    applyK(s, 0, P->v1, P->v2);
    for (int64_t i = 0; i < nv; i++) P->v2[i] *= P->w0[i];
    applyGt(s, P->v2, s->pt2, 0);
    for (int64_t e = 0; e < np; e++) P->fr[e] = (float)s->pt2[e];
    plsolve(P, P->fr, P->fz, rtol, 200);
    double mean = 0.0;
    for (int64_t e = 0; e < np; e++) { z[e] = -(double)P->fz[e]; mean += z[e]; }
    mean /= (double)np;
    for (int64_t e = 0; e < np; e++) z[e] -= mean;
}

static double wtime(void) {
    struct timespec t;
    clock_gettime(CLOCK_MONOTONIC, &t);
    return (double)t.tv_sec + 1e-9 * (double)t.tv_nsec;
}

/* Seconds per iteration of the two Krylov loops the solve spends its time in,
 * on this mesh: out[0] one multigrid-preconditioned CG iteration of the
 * velocity operator (K apply + V-cycle + vector updates), out[1] one CG
 * iteration of the BFBt pressure Laplacian (L apply + pressure V-cycle), or 0
 * without BFBt.  n_vel / n_l iterations are run from a fixed right-hand side;
 * deg is the Chebyshev degree of the velocity smoother. */
void uwo_sys_time_iterations(uwo_sys* s, int n_vel, int n_l, int deg, double* out) {
    for (int64_t i = 0; i < s->nv; i++) s->u1[i] = s->L[0].bc[i] ? 0.0 : sin(0.37 * (double)i);
    double t0 = wtime();
    int it = pcg(s, s->u1, s->u2, 1e-300, n_vel, deg);
    out[0] = (wtime() - t0) / (double)(it < 0 ? -it : (it > 0 ? it : 1));
    out[1] = 0.0;
    if (s->pmg && n_l > 0) {
        struct pmg_s* P = s->pmg;
        for (int64_t e = 0; e < s->np; e++) P->fr[e] = (float)sin(0.53 * (double)e);
        int before = P->its;
        t0 = wtime();
        plsolve(P, P->fr, P->fz, 0.0, n_l);
        out[1] = (wtime() - t0) / (double)(P->its - before > 0 ? P->its - before : 1);
        P->its = before;
    }
}

/* Schur preconditioner of the next uwo_sys_finish / solve: pc 0 = the Uzawa
 * term (the reference's "uw"), 1 = weighted scaled BFBt with a pressure
 * multigrid of Chebyshev degree deg and L-solves to rtol. */
void uwo_sys_set_schur_pc(uwo_sys* s, int pc, int deg, double rtol) {
    s->schur_pc = pc;
    s->pc_deg = deg > 0 ? deg : 2;
    s->pc_rtol = rtol > 0.0 ? rtol : 3e-2;
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
                if (s->pmg) bfbt_apply(s, s->pmg, s->V[j], s->Z[j], s->pc_rtol);
                else for (int64_t e = 0; e < np; e++) s->Z[j][e] = -s->V[j][e] / s->shat[e];
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
    stats[5] = s->pmg ? s->pmg->its : 0;
    if (s->pmg) s->pmg->its = 0;
    return rc;
}
