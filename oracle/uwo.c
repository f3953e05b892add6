/*
 * uwo.c -- CPU oracle for the particle-in-cell Stokes path.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is a plain-C FP64 restatement of the
 * reference algorithms.  It is the checker for the CUDA library and the CPU
 * baseline that the benchmark times; no product code path may call it.
 *
 * Compile with -ffp-contract=off: every expression below is evaluated as
 * separate IEEE multiplies and adds, in the order the reference writes them,
 * so that particle coordinates, local coordinates and element ownership are
 * bit-for-bit reproducible.
 *
 * Citations are to files of the underworld2 source tree, with
 *   L/ = src/underworld/libUnderworld/
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#define UWO_EPS 1e-12 /* Num_Epsilon: L/StGermain/Base/Foundation/src/Numerics.c:17 */

/* Num_Approx: L/StGermain/Base/Foundation/src/Numerics.c:20-22 */
static int num_approx(double var, double val) {
    return var >= val - UWO_EPS && var <= val + UWO_EPS;
}

/* ------------------------------------------------------------------------ */
/* Mesh description.  A regular Cartesian mesh of Q1 (order 1) or Q2 (order  */
/* 2) elements; node coordinates per axis follow CartesianGenerator_CalcGeom */
/* (L/StgDomain/Mesh/src/CartesianGenerator.c:2003-2036, contact depth 0):   */
/*   x_i = min + (i / (n-1)) * (max - min), ends pinned to min and max.      */
/* ------------------------------------------------------------------------ */
typedef struct {
    int dim;
    int order;      /* 1 = Q1, 2 = Q2 */
    int res[3];     /* elements per axis */
    double minc[3];
    double maxc[3];
} uwo_mesh;

int uwo_nodes_per_axis(const uwo_mesh* m, int d) { return m->res[d] * m->order + 1; }

void uwo_axis_coords(const uwo_mesh* m, int d, double* out) {
    int n = uwo_nodes_per_axis(m, d);
    double steps = m->maxc[d] - m->minc[d];
    for (int i = 0; i < n; i++) {
        if (i <= 0) out[i] = m->minc[d];
        else if (i >= n - 1) out[i] = m->maxc[d];
        else out[i] = m->minc[d] + ((double)i / (double)(n - 1)) * steps;
    }
}

int uwo_el_nodes(const uwo_mesh* m) {
    int k = m->order + 1;
    return m->dim == 2 ? k * k : k * k * k;
}

/* Element -> node incidence, local order x fastest
 * (L/StgDomain/Mesh/src/CartesianGenerator.c:743-800 for Q1,
 *  L/StgFEM/Discretisation/src/C2Generator.c:147-250 for Q2). */
void uwo_element_nodes(const uwo_mesh* m, int64_t el, int64_t* nodes) {
    int64_t ex = el % m->res[0];
    int64_t ey = (el / m->res[0]) % m->res[1];
    int64_t ez = m->dim == 3 ? el / ((int64_t)m->res[0] * m->res[1]) : 0;
    int64_t nx = uwo_nodes_per_axis(m, 0), ny = uwo_nodes_per_axis(m, 1);
    int k = m->order + 1, c = 0;
    int kz = m->dim == 3 ? k : 1;
    for (int a = 0; a < kz; a++)
        for (int b = 0; b < k; b++)
            for (int i = 0; i < k; i++) {
                int64_t ix = ex * m->order + i, iy = ey * m->order + b, iz = ez * m->order + a;
                nodes[c++] = ix + nx * (iy + ny * iz);
            }
}

static void node_xyz(const uwo_mesh* m, const double* const* ax, int64_t node, double* x) {
    int64_t nx = uwo_nodes_per_axis(m, 0), ny = uwo_nodes_per_axis(m, 1);
    x[0] = ax[0][node % nx];
    x[1] = ax[1][(node / nx) % ny];
    if (m->dim == 3) x[2] = ax[2][node / (nx * ny)];
}

/* ------------------------------------------------------------------------ */
/* Shape functions                                                           */
/* ------------------------------------------------------------------------ */
/* L/StgFEM/Discretisation/src/BilinearElementType.c:179-211 */
static void q1_2d(const double* l, double* N, double (*G)[27]) {
    double xi = l[0], eta = l[1];
    N[0] = 0.25 * (1.0 - xi) * (1.0 - eta);
    N[1] = 0.25 * (1.0 + xi) * (1.0 - eta);
    N[2] = 0.25 * (1.0 - xi) * (1.0 + eta);
    N[3] = 0.25 * (1.0 + xi) * (1.0 + eta);
    if (!G) return;
    G[0][0] = -(0.25 * (1.0 - eta));
    G[0][1] = 0.25 * (1.0 - eta);
    G[0][3] = 0.25 * (1.0 + eta);
    G[0][2] = -(0.25 * (1.0 + eta));
    G[1][0] = -(0.25 * (1.0 - xi));
    G[1][1] = -(0.25 * (1.0 + xi));
    G[1][3] = 0.25 * (1.0 + xi);
    G[1][2] = 0.25 * (1.0 - xi);
}

/* L/StgFEM/Discretisation/src/TrilinearElementType.c:215-274 */
static void q1_3d(const double* l, double* N, double (*G)[27]) {
    double xi = l[0], eta = l[1], zeta = l[2];
    N[0] = 0.125 * (1.0 - xi) * (1.0 - eta) * (1.0 - zeta);
    N[2] = 0.125 * (1.0 - xi) * (1.0 + eta) * (1.0 - zeta);
    N[3] = 0.125 * (1.0 + xi) * (1.0 + eta) * (1.0 - zeta);
    N[1] = 0.125 * (1.0 + xi) * (1.0 - eta) * (1.0 - zeta);
    N[4] = 0.125 * (1.0 - xi) * (1.0 - eta) * (1.0 + zeta);
    N[6] = 0.125 * (1.0 - xi) * (1.0 + eta) * (1.0 + zeta);
    N[7] = 0.125 * (1.0 + xi) * (1.0 + eta) * (1.0 + zeta);
    N[5] = 0.125 * (1.0 + xi) * (1.0 - eta) * (1.0 + zeta);
    if (!G) return;
    G[0][0] = -(0.125 * (1.0 - eta) * (1.0 - zeta));
    G[0][2] = -(0.125 * (1.0 + eta) * (1.0 - zeta));
    G[0][3] = 0.125 * (1.0 + eta) * (1.0 - zeta);
    G[0][1] = 0.125 * (1.0 - eta) * (1.0 - zeta);
    G[0][4] = -(0.125 * (1.0 - eta) * (1.0 + zeta));
    G[0][6] = -(0.125 * (1.0 + eta) * (1.0 + zeta));
    G[0][7] = 0.125 * (1.0 + eta) * (1.0 + zeta);
    G[0][5] = 0.125 * (1.0 - eta) * (1.0 + zeta);
    G[1][0] = -(0.125 * (1.0 - xi) * (1.0 - zeta));
    G[1][2] = 0.125 * (1.0 - xi) * (1.0 - zeta);
    G[1][3] = 0.125 * (1.0 + xi) * (1.0 - zeta);
    G[1][1] = -(0.125 * (1.0 + xi) * (1.0 - zeta));
    G[1][4] = -(0.125 * (1.0 - xi) * (1.0 + zeta));
    G[1][6] = 0.125 * (1.0 - xi) * (1.0 + zeta);
    G[1][7] = 0.125 * (1.0 + xi) * (1.0 + zeta);
    G[1][5] = -(0.125 * (1.0 + xi) * (1.0 + zeta));
    G[2][0] = -0.125 * (1.0 - xi) * (1.0 - eta);
    G[2][2] = -0.125 * (1.0 - xi) * (1.0 + eta);
    G[2][3] = -0.125 * (1.0 + xi) * (1.0 + eta);
    G[2][1] = -0.125 * (1.0 + xi) * (1.0 - eta);
    G[2][4] = 0.125 * (1.0 - xi) * (1.0 - eta);
    G[2][6] = 0.125 * (1.0 - xi) * (1.0 + eta);
    G[2][7] = 0.125 * (1.0 + xi) * (1.0 + eta);
    G[2][5] = 0.125 * (1.0 + xi) * (1.0 - eta);
}

/* L/StgFEM/Discretisation/src/Biquadratic.c:138-200 */
static void q2_2d(const double* l, double* N, double (*G)[27]) {
    double xi = l[0], eta = l[1];
    {
        double a0 = xi - 1.0, b0 = eta - 1.0;
        double a1 = 1.0 - xi * xi, b1 = 1.0 - eta * eta;
        double a2 = xi + 1.0, b2 = eta + 1.0;
        double m0 = 0.5 * xi, m1 = 0.5 * eta, m2 = 0.25 * xi * eta;
        N[0] = m2 * a0 * b0; N[1] = m1 * a1 * b0; N[2] = m2 * a2 * b0;
        N[3] = m0 * a0 * b1; N[4] = a1 * b1;      N[5] = m0 * a2 * b1;
        N[6] = m2 * a0 * b2; N[7] = m1 * a1 * b2; N[8] = m2 * a2 * b2;
    }
    if (!G) return;
    {
        double a0 = xi - 1.0, b0 = eta - 1.0;
        double a1 = xi + 1.0, b1 = eta + 1.0;
        double a2 = 2.0 * xi - 1.0, b2 = 2.0 * eta - 1.0;
        double a3 = 2.0 * xi + 1.0, b3 = 2.0 * eta + 1.0;
        double a4 = 1.0 - xi * xi, b4 = 1.0 - eta * eta;
        double m0 = 0.25 * xi, m1 = 0.25 * eta, m2 = -xi * eta;
        G[0][0] = m1 * a2 * b0; G[0][2] = m1 * a3 * b0;
        G[0][6] = m1 * a2 * b1; G[0][8] = m1 * a3 * b1;
        G[1][0] = m0 * a0 * b2; G[1][2] = m0 * a1 * b2;
        G[1][6] = m0 * a0 * b3; G[1][8] = m0 * a1 * b3;
        G[0][1] = m2 * b0; G[0][7] = m2 * b1;
        G[0][3] = 0.5 * a2 * b4; G[0][5] = 0.5 * a3 * b4;
        G[1][1] = 0.5 * a4 * b2; G[1][7] = 0.5 * a4 * b3;
        G[1][3] = m2 * a0; G[1][5] = m2 * a1;
        G[0][4] = -2.0 * xi * b4;
        G[1][4] = -2.0 * eta * a4;
    }
}

/* Triquadratic basis (L/StgFEM/Discretisation/src/Triquadratic.c:193-400).
 * Node n = a + 3b + 9c; basis = m * A_a * B_b * C_c with A = {xi-1, 1-xi^2,
 * xi+1} (B, C likewise) and m the reference's m0..m6: the product of the
 * 1/2-scaled coordinates of the axes on which the node is a corner node.  A
 * derivative swaps one factor for {xi-1/2, -2xi, xi+1/2} and keeps the m
 * factor of the other two axes.  Products are formed in the reference's order. */
static void q2_3d(const double* l, double* N, double (*G)[27]) {
    double xi = l[0], eta = l[1], zeta = l[2];
    double A[3] = {xi - 1.0, 1.0 - xi * xi, xi + 1.0};
    double B[3] = {eta - 1.0, 1.0 - eta * eta, eta + 1.0};
    double C[3] = {zeta - 1.0, 1.0 - zeta * zeta, zeta + 1.0};
    double dA[3] = {xi - 0.5, -2.0 * xi, xi + 0.5};
    double dB[3] = {eta - 0.5, -2.0 * eta, eta + 0.5};
    double dC[3] = {zeta - 0.5, -2.0 * zeta, zeta + 0.5};
    double m0 = 0.5 * xi, m1 = 0.5 * eta, m2 = 0.5 * zeta;
    double m3 = 0.25 * xi * eta, m4 = 0.25 * xi * zeta, m5 = 0.25 * eta * zeta;
    double m6 = 0.125 * xi * eta * zeta;
    /* m for the corner-axis set (x: 4, y: 2, z: 1) */
    double mfull[8] = {1.0, m2, m1, m5, m0, m4, m3, m6};
    for (int n = 0; n < 27; n++) {
        int a = n % 3, b = (n / 3) % 3, c = n / 9;
        int ex = a != 1, ey = b != 1, ez = c != 1;
        int sel = ex * 4 + ey * 2 + ez;
        N[n] = sel ? mfull[sel] * A[a] * B[b] * C[c] : A[a] * B[b] * C[c];
        if (!G) continue;
        double myz = ey && ez ? m5 : ey ? m1 : ez ? m2 : 0.0;
        double mxz = ex && ez ? m4 : ex ? m0 : ez ? m2 : 0.0;
        double mxy = ex && ey ? m3 : ex ? m0 : ey ? m1 : 0.0;
        G[0][n] = (ey || ez) ? dA[a] * myz * B[b] * C[c] : dA[a] * B[b] * C[c];
        G[1][n] = (ex || ez) ? dB[b] * mxz * A[a] * C[c] : dB[b] * A[a] * C[c];
        G[2][n] = (ex || ey) ? dC[c] * mxy * A[a] * B[b] : dC[c] * A[a] * B[b];
    }
}

void uwo_shape(int dim, int order, const double* xi, double* N, double* G /* [3][27] */) {
    double (*GG)[27] = (double (*)[27])G;
    if (order == 1) { if (dim == 2) q1_2d(xi, N, GG); else q1_3d(xi, N, GG); }
    else { if (dim == 2) q2_2d(xi, N, GG); else q2_3d(xi, N, GG); }
}

/* Pressure bases: dQ0 (L/StgFEM/Discretisation/src/ConstantElementType.c:131)
 * and dPc1 (BilinearInnerElType.c:169-179, TrilinearInnerElType.c:202-215). */
int uwo_pressure_nodes(int dim, int porder) { return porder == 0 ? 1 : (dim == 2 ? 3 : 4); }
void uwo_pressure_shape(int dim, int porder, const double* l, double* M) {
    if (porder == 0) { M[0] = 1.0; return; }
    if (dim == 2) {
        double xi = l[0], eta = l[1];
        M[0] = -xi - 0.5 * eta + 0.25;
        M[1] = xi - 0.5 * eta + 0.25;
        M[2] = eta + 0.5;
    } else {
        double xi = l[0], eta = l[1], zeta = l[2], fac = 1.0 / 9.0;
        M[0] = fac * (-4.0 * xi - 20.0 * eta + 12.0 * zeta + 3.0);
        M[1] = fac * (16.0 * xi - 64.0 * eta + 60.0 * zeta + 6.0);
        M[2] = fac * (36.0 * eta - 36.0 * zeta);
        M[3] = fac * (-12.0 * xi + 48.0 * eta - 36.0 * zeta);
    }
}

/* ------------------------------------------------------------------------ */
/* Park-Miller minimal standard RNG with Schrage's method                    */
/* (L/StgDomain/Swarm/src/Random.c:23-53).                                   */
/* ------------------------------------------------------------------------ */
static const int64_t PM_M = 2147483647, PM_A = 16807, PM_Q = 127773, PM_R = 2836;
static const int64_t PM_MASK = 123459876;

int64_t uwo_rng_seed(int64_t seed) { return seed ^ PM_MASK; }

static double rng_next(int64_t* s) {
    int64_t tmp = *s / PM_Q;
    *s = PM_A * (*s - tmp * PM_Q) - PM_R * tmp;
    if (*s < 0) *s += PM_M;
    return (double)*s;
}

/* Swarm_Random_Random_WithMinMax (Random.c:51-53) */
static double rng_minmax(int64_t* s, double mn, double mx) {
    return (mx - mn) * rng_next(s) / (double)PM_M + mn;
}

/* Local -> global through the element basis (L/StgFEM/Discretisation/src/FeMesh.c:333-360). */
static void local_to_global(const uwo_mesh* m, const double* const* ax, int64_t el,
                            const double* xi, double* x) {
    int64_t nodes[27];
    double N[27], vert[3];
    int nen = uwo_el_nodes(m);
    uwo_element_nodes(m, el, nodes);
    uwo_shape(m->dim, m->order, xi, N, NULL);
    for (int d = 0; d < m->dim; d++) x[d] = 0.0;
    for (int n = 0; n < nen; n++) {
        node_xyz(m, ax, nodes[n], vert);
        for (int d = 0; d < m->dim; d++) x[d] += N[n] * vert[d];
    }
}

/* PerCellRandomLayout: cells in order, particles in order, dims in order,
 * one global stream (L/StgFEM/Utils/src/MeshParticleLayout.c:194-230,
 * L/StgDomain/Swarm/src/PerCellParticleLayout.c:117-140).  Returns the RNG
 * state after the last draw. */
int64_t uwo_layout_random(const uwo_mesh* m, const double* ax0, const double* ax1, const double* ax2,
                          int ppc, int64_t state, double* coords) {
    const double* ax[3] = {ax0, ax1, ax2};
    int64_t nel = (int64_t)m->res[0] * m->res[1] * (m->dim == 3 ? m->res[2] : 1);
    double xi[3];
    for (int64_t e = 0; e < nel; e++)
        for (int p = 0; p < ppc; p++) {
            for (int d = 0; d < m->dim; d++) xi[d] = rng_minmax(&state, -1.0, 1.0);
            local_to_global(m, ax, e, xi, coords + (e * ppc + p) * m->dim);
        }
    return state;
}

/* ------------------------------------------------------------------------ */
/* Element search                                                            */
/* ------------------------------------------------------------------------ */
/* Mesh_RegularAlgorithms_SearchElements
 * (L/StgDomain/Mesh/src/Mesh_RegularAlgorithms.c:174-205); sep from :154. */
int uwo_search_element(const uwo_mesh* m, const double* p, int64_t* el) {
    int64_t inds[3] = {0, 0, 0};
    for (int d = 0; d < m->dim; d++) {
        double sep = (m->maxc[d] - m->minc[d]) / m->res[d];
        if (num_approx(p[d] - m->maxc[d], 0.0)) inds[d] = m->res[d] - 1;
        else if (p[d] < m->minc[d] || p[d] > m->maxc[d]) return 0;
        else {
            double integer;
            double out = (p[d] - m->minc[d]) / sep;
            double frac = modf(out, &integer);
            inds[d] = (int64_t)(unsigned)integer;
            if (inds[d] > 0 && num_approx(frac, 0.0)) inds[d]--;
        }
    }
    *el = inds[0] + (int64_t)m->res[0] * (inds[1] + (int64_t)m->res[1] * inds[2]);
    return 1;
}

/* _ElementCellLayout_CellOf (L/StgDomain/Swarm/src/ElementCellLayout.c:291-320):
 * domain filter, then the regular search.  Returns n_el when outside. */
int64_t uwo_cell_of(const uwo_mesh* m, const double* p) {
    int64_t nel = (int64_t)m->res[0] * m->res[1] * (m->dim == 3 ? m->res[2] : 1);
    for (int d = 0; d < m->dim; d++)
        if (p[d] < m->minc[d] || p[d] > m->maxc[d]) return nel;
    int64_t el;
    if (!uwo_search_element(m, p, &el)) return nel;
    return el;
}

/* TensorArray_SolveSystem (L/StgDomain/Geometry/src/TensorMath.c:959-1010) */
static void solve_system(const double* t, double* s, const double* r, int dim) {
    if (dim == 3) {
        double det = +t[0] * (t[4] * t[8] - t[7] * t[5])
                     - t[1] * (t[3] * t[8] - t[5] * t[6])
                     + t[2] * (t[3] * t[7] - t[4] * t[6]);
        s[0] = (r[0] * (t[4] * t[8] - t[7] * t[5])
                - t[1] * (r[1] * t[8] - t[5] * r[2])
                + t[2] * (r[1] * t[7] - t[4] * r[2])) / det;
        s[1] = (t[0] * (r[1] * t[8] - r[2] * t[5])
                - r[0] * (t[3] * t[8] - t[5] * t[6])
                + t[2] * (t[3] * r[2] - r[1] * t[6])) / det;
        s[2] = (t[0] * (t[4] * r[2] - t[7] * r[1])
                - t[1] * (t[3] * r[2] - r[1] * t[6])
                + r[0] * (t[3] * t[7] - t[4] * t[6])) / det;
    } else {
        double det = t[0] * t[3] - t[2] * t[1];
        s[0] = (r[0] * t[3] - t[1] * r[1]) / det;
        s[1] = (r[1] * t[0] - t[2] * r[0]) / det;
    }
}

/* Newton-Raphson global -> local (L/StgFEM/Discretisation/src/ElementType.c:177-301):
 * start at the centre, tolerance 1e-4 on the increment, at most 100
 * iterations, failure marks xi[0] = 1.1.  Returns the iteration count. */
int uwo_global_to_local(const uwo_mesh* m, const double* ax0, const double* ax1, const double* ax2,
                        int64_t el, const double* x, double* xi) {
    const double* ax[3] = {ax0, ax1, ax2};
    int64_t nodes[27];
    double N[27], G[3][27], v[3];
    int dim = m->dim, nen = uwo_el_nodes(m);
    uwo_element_nodes(m, el, nodes);
    for (int d = 0; d < dim; d++) xi[d] = 0.0;
    for (int it = 0; it < 100; it++) {
        double J[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0}, r[3] = {0, 0, 0}, dxi[3];
        uwo_shape(dim, m->order, xi, N, &G[0][0]);
        for (int n = 0; n < nen; n++) {
            node_xyz(m, ax, nodes[n], v);
            if (dim == 2) {
                J[0] += G[0][n] * v[0];
                J[1] += G[1][n] * v[0];
                J[2] += G[0][n] * v[1];
                J[3] += G[1][n] * v[1];
                r[0] -= N[n] * v[0];
                r[1] -= N[n] * v[1];
            } else {
                J[0] += G[0][n] * v[0];
                J[1] += G[1][n] * v[0];
                J[3] += G[0][n] * v[1];
                J[4] += G[1][n] * v[1];
                r[0] -= N[n] * v[0];
                r[1] -= N[n] * v[1];
                J[2] += G[2][n] * v[0];
                J[5] += G[2][n] * v[1];
                J[6] += G[0][n] * v[2];
                J[7] += G[1][n] * v[2];
                J[8] += G[2][n] * v[2];
                r[2] -= N[n] * v[2];
            }
        }
        r[0] += x[0];
        r[1] += x[1];
        if (dim == 3) r[2] += x[2];
        solve_system(J, dxi, r, dim);
        xi[0] += dxi[0];
        xi[1] += dxi[1];
        if (dim == 3) xi[2] += dxi[2];
        double mr = fabs(dxi[0]);
        if (mr < fabs(dxi[1])) mr = fabs(dxi[1]);
        if (dim == 3 && mr < fabs(dxi[2])) mr = fabs(dxi[2]);
        if (mr < 0.0001) return it + 1;
    }
    xi[0] = 1.1;
    return 100;
}

/* ------------------------------------------------------------------------ */
/* Cell tables: particle index lists per element, built by the layout in     */
/* particle order and edited by the owner update.                            */
/* ------------------------------------------------------------------------ */

/* Swarm_UpdateAllParticleOwners / Swarm_UpdateParticleOwner /
 * Swarm_RemoveParticleFromCell (L/StgDomain/Swarm/src/SwarmClass.c:947-1015).
 * Tables are fixed-capacity slabs: tbl[c*cap + k], cnt[c].  Returns the
 * number of particles that left the domain, or -1 when a slab overflows. */
int64_t uwo_update_owners(const uwo_mesh* m, int64_t np, const double* coords, int32_t* owner,
                          int32_t* tbl, int32_t* cnt, int cap) {
    int64_t nel = (int64_t)m->res[0] * m->res[1] * (m->dim == 3 ? m->res[2] : 1);
    int64_t lost = 0;
    for (int64_t p = 0; p < np; p++) {
        int64_t nc = uwo_cell_of(m, coords + p * m->dim);
        int64_t oc = owner[p];
        if (nc == oc) continue;
        if (oc < nel) {
            int32_t* t = tbl + oc * cap;
            int k = 0;
            while (k < cnt[oc] && t[k] != p) k++;
            t[k] = t[cnt[oc] - 1];
            cnt[oc]--;
        }
        if (nc == nel) { owner[p] = (int32_t)nel; lost++; }
        else {
            if (cnt[nc] >= cap) return -1;
            tbl[nc * cap + cnt[nc]] = (int32_t)p;
            cnt[nc]++;
            owner[p] = (int32_t)nc;
        }
    }
    return lost;
}

/* ------------------------------------------------------------------------ */
/* Discrete Voronoi cell weights (L/PICellerator/Weights/src/DVCWeights.c).  */
/* ------------------------------------------------------------------------ */
typedef struct { int p, done; int nb[6]; double x, y, z; } dvc_cell;
typedef struct { int nclaimed, nbound; int* claimed; int* bound; } dvc_chain;

/* _DVCWeights_ConstructGrid / _DVCWeights_ConstructGrid2D (:491-586):
 * neighbour order S, N, E, W, U, D; centres accumulated by repeated adds. */
static void dvc_grid(int dim, int nx, int ny, int nz, dvc_cell* cells) {
    int l = nx, mm = ny, n = dim == 3 ? nz : 1;
    int tot = l * mm * n;
    for (int i = 0; i < tot; i++) {
        for (int k = 0; k < 6; k++) cells[i].nb[k] = -2;
        cells[i].p = -1; cells[i].done = 0;
        cells[i].x = cells[i].y = cells[i].z = 0.0;
    }
    for (int k = 0; k < n; k++)
        for (int i = 0; i < l * (mm - 1); i++) {
            cells[i + k * l * mm].nb[1] = i + k * l * mm + l;     /* N */
            cells[i + l + k * l * mm].nb[0] = i + k * l * mm;     /* S */
        }
    for (int k = 0; k < n - 1; k++)
        for (int i = 0; i < l * mm; i++) {
            cells[i + k * l * mm].nb[4] = i + k * l * mm + l * mm; /* U */
            cells[i + k * l * mm + l * mm].nb[5] = i + k * l * mm; /* D */
        }
    double dx = (1.0 - -1.0) / l, dy = (1.0 - -1.0) / mm, dz = (1.0 - -1.0) / n;
    double X, Y, Z = -1.0 - dz / 2.0;
    for (int k = 0; k < n; k++) {
        Z = Z + dz;
        Y = -1.0 - dy / 2.0;
        for (int j = 0; j < mm; j++) {
            Y = Y + dy;
            X = -1.0 - dx / 2.0;
            for (int i = 0; i < l; i++) {
                X = X + dx;
                int c = i + l * j + k * l * mm;
                cells[c].x = X; cells[c].y = Y; cells[c].z = dim == 3 ? Z : 0.0;
                if (i != l - 1) {
                    cells[c].nb[2] = c + 1;      /* E */
                    cells[c + 1].nb[3] = c;      /* W */
                }
            }
        }
    }
}

/* _DVCWeights_UpdateBchain(2D) (:388-486) */
static void dvc_update_bchain(dvc_chain* ch, dvc_cell* cells, int pi, int nnb) {
    dvc_chain* b = &ch[pi];
    int count = 0;
    for (int i = 0; i < b->nclaimed; i++) {
        int c0 = b->claimed[i];
        for (int k = 0; k < nnb; k++) {
            int c1 = cells[c0].nb[k];
            if (c1 != -2 && cells[c1].p != pi && cells[c1].done != 1) {
                b->bound[count++] = c1;
                cells[c1].done = 1;
            }
        }
    }
    b->nbound = count;
    for (int i = 0; i < count; i++) cells[b->bound[i]].done = 0;
}

/* _DVCWeights_DistanceTest(2D) (:595-600) */
static double dvc_dist_test(int dim, double x0, double y0, double z0, double x1, double y1, double z1,
                            double x2, double y2, double z2) {
    if (dim == 2) return (x1 + x2 - x0 - x0) * (x1 - x2) + (y1 + y2 - y0 - y0) * (y1 - y2);
    return (x1 + x2 - x0 - x0) * (x1 - x2) + (y1 + y2 - y0 - y0) * (y1 - y2) + (z1 + z2 - z0 - z0) * (z1 - z2);
}

/* _DVCWeights_ClaimCells(2D) (:256-365) */
static void dvc_claim(int dim, dvc_chain* ch, dvc_cell* cells, const double* px, int pi) {
    dvc_chain* b = &ch[pi];
    int count = 0;
    for (int i = 0; i < b->nbound; i++) {
        int c0 = b->bound[i];
        if (cells[c0].p == -1) {
            b->claimed[count++] = c0;
            cells[c0].p = pi;
        } else if (cells[c0].p != pi) {
            int q = cells[c0].p;
            double d = dvc_dist_test(dim, cells[c0].x, cells[c0].y, cells[c0].z,
                                     px[q * 3 + 0], px[q * 3 + 1], px[q * 3 + 2],
                                     px[pi * 3 + 0], px[pi * 3 + 1], px[pi * 3 + 2]);
            if (d > 0.0) {
                b->claimed[count++] = c0;
                cells[c0].p = pi;
            }
        }
    }
    b->nclaimed = count;
}

/* One element: _DVCWeights_Calculate2D/3D (:772-927) with CreateVoronoi
 * (:676-770) and GetCentroids (:198-254).  xi[nump*dim] in, centroid and
 * weight out.  Returns the number of growth rounds. */
int uwo_dvc_element(int dim, int res, int nump, const double* xi, double* cxi, double* w) {
    int nx = res, ny = res, nz = dim == 3 ? res : 1;
    int tot = nx * ny * nz, nnb = dim == 3 ? 6 : 4;
    dvc_cell* cells = (dvc_cell*)malloc(sizeof(dvc_cell) * tot);
    dvc_chain* ch = (dvc_chain*)malloc(sizeof(dvc_chain) * nump);
    int* pool = (int*)malloc(sizeof(int) * (size_t)nump * 2 * (tot + 1));
    double* px = (double*)calloc((size_t)nump * 3, sizeof(double));
    dvc_grid(dim, nx, ny, nz, cells);
    double dx = (1.0 - -1.0) / nx, dy = (1.0 - -1.0) / ny, dz = (1.0 - -1.0) / nz;
    double da = dim == 3 ? dx * dy * dz : dx * dy;
    for (int i = 0; i < nump; i++) {
        ch[i].claimed = pool + (size_t)i * 2 * (tot + 1);
        ch[i].bound = ch[i].claimed + tot + 1;
        for (int d = 0; d < dim; d++) px[i * 3 + d] = xi[i * dim + d];
    }
    for (int i = 0; i < nump; i++) {
        int k = (int)((px[i * 3 + 0] - -1.0) / dx);
        int j = (int)((px[i * 3 + 1] - -1.0) / dy);
        int l = dim == 3 ? (int)((px[i * 3 + 2] - -1.0) / dz) : 0;
        if (k == nx) k--;
        if (j == ny) j--;
        if (dim == 3 && l == nz) l--;
        int c = k + j * nx + l * nx * ny;
        cells[c].p = i;
        ch[i].nclaimed = 1;
        ch[i].nbound = 0;
        ch[i].claimed[0] = c;
        dvc_update_bchain(ch, cells, i, nnb);
    }
    int rounds = 0, claimed = 1;
    while (claimed != 0) {
        claimed = 0;
        rounds++;
        for (int i = 0; i < nump; i++) {
            dvc_claim(dim, ch, cells, px, i);
            claimed += ch[i].nclaimed;
            dvc_update_bchain(ch, cells, i, nnb);
        }
    }
    int* count = (int*)calloc(nump, sizeof(int));
    double* c3 = (double*)calloc((size_t)nump * 3, sizeof(double));
    for (int i = 0; i < tot; i++) {
        int p = cells[i].p;
        c3[p * 3 + 0] += cells[i].x;
        c3[p * 3 + 1] += cells[i].y;
        if (dim == 3) c3[p * 3 + 2] += cells[i].z;
        count[p]++;
    }
    for (int i = 0; i < nump; i++) {
        w[i] = count[i] * da;
        for (int d = 0; d < dim; d++) {
            double v = c3[i * 3 + d];
            if (count[i] != 0) v /= count[i];
            cxi[i * dim + d] = v;
        }
    }
    free(count); free(c3); free(cells); free(ch); free(pool); free(px);
    return rounds;
}

/* ------------------------------------------------------------------------ */
/* Coincident mapping + DVC over all cells (L/PICellerator/MaterialPoints/   */
/* src/CoincidentMapper.c:76-125, L/PICellerator/Weights/src/                */
/* WeightsCalculator.c:114-150).  Integration point k of cell c is the       */
/* material particle tbl[c*cap+k]; outputs are indexed by particle.          */
/* ------------------------------------------------------------------------ */
void uwo_pic_map(const uwo_mesh* m, const double* ax0, const double* ax1, const double* ax2,
                 const double* coords, const int32_t* tbl, const int32_t* cnt, int cap,
                 int64_t c0, int64_t c1, int dvc_res, double* ip_xi, double* ip_w) {
    int dim = m->dim;
#pragma omp parallel
    {
        double* xi = (double*)malloc(sizeof(double) * cap * dim);
        double* cx = (double*)malloc(sizeof(double) * cap * dim);
        double* w = (double*)malloc(sizeof(double) * cap);
#pragma omp for schedule(dynamic, 16)
        for (int64_t c = c0; c < c1; c++) {
            int n = cnt[c];
            for (int k = 0; k < n; k++) {
                int32_t p = tbl[c * cap + k];
                uwo_global_to_local(m, ax0, ax1, ax2, c, coords + (int64_t)p * dim, xi + k * dim);
            }
            if (n > 0) uwo_dvc_element(dim, dvc_res, n, xi, cx, w);
            for (int k = 0; k < n; k++) {
                int32_t p = tbl[c * cap + k];
                for (int d = 0; d < dim; d++) ip_xi[(int64_t)p * dim + d] = cx[k * dim + d];
                ip_w[p] = w[k];
            }
        }
        free(xi); free(cx); free(w);
    }
}

/* ------------------------------------------------------------------------ */
/* Element terms                                                             */
/* ------------------------------------------------------------------------ */
/* ElementType_ShapeFunctionsGlobalDerivs (ElementType.c:305-447) */
static double global_derivs(const uwo_mesh* m, const double* const* ax, const int64_t* nodes,
                            const double* xi, double* N, double (*GNx)[27]) {
    double G[3][27], v[3], jac[3][3] = {{0}}, D = 0.0;
    int dim = m->dim, nen = uwo_el_nodes(m);
    uwo_shape(dim, m->order, xi, N, &G[0][0]);
    for (int n = 0; n < nen; n++) {
        node_xyz(m, ax, nodes[n], v);
        for (int i = 0; i < dim; i++)
            for (int j = 0; j < dim; j++) jac[i][j] = jac[i][j] + G[i][n] * v[j];
    }
    double inv[3][3];
    if (dim == 2) {
        D = jac[0][0] * jac[1][1] - jac[0][1] * jac[1][0];
        inv[0][0] = jac[1][1] / D; inv[1][1] = jac[0][0] / D;
        inv[0][1] = -jac[0][1] / D; inv[1][0] = -jac[1][0] / D;
    } else {
        D = jac[0][0] * (jac[1][1] * jac[2][2] - jac[1][2] * jac[2][1])
            - jac[0][1] * (jac[1][0] * jac[2][2] - jac[1][2] * jac[2][0])
            + jac[0][2] * (jac[1][0] * jac[2][1] - jac[1][1] * jac[2][0]);
        double cof[3][3];
        cof[0][0] = jac[1][1] * jac[2][2] - jac[1][2] * jac[2][1];
        cof[1][0] = -(jac[1][0] * jac[2][2] - jac[1][2] * jac[2][0]);
        cof[2][0] = jac[1][0] * jac[2][1] - jac[1][1] * jac[2][0];
        cof[0][1] = -(jac[0][1] * jac[2][2] - jac[0][2] * jac[2][1]);
        cof[1][1] = jac[0][0] * jac[2][2] - jac[0][2] * jac[2][0];
        cof[2][1] = -(jac[0][0] * jac[2][1] - jac[0][1] * jac[2][0]);
        cof[0][2] = jac[0][1] * jac[1][2] - jac[0][2] * jac[1][1];
        cof[1][2] = -(jac[0][0] * jac[1][2] - jac[0][2] * jac[1][0]);
        cof[2][2] = jac[0][0] * jac[1][1] - jac[0][1] * jac[1][0];
        for (int i = 0; i < 3; i++)
            for (int j = 0; j < 3; j++) inv[i][j] = cof[i][j] / D;
    }
    for (int dx = 0; dx < dim; dx++)
        for (int n = 0; n < nen; n++) {
            double s = 0.0;
            for (int dxi = 0; dxi < dim; dxi++) s = s + G[dxi][n] * inv[dx][dxi];
            GNx[dx][n] = s;
        }
    return D;
}

/* K_e for one element from a list of quadrature points (xi, weight, eta):
 * K_e = sum_q w_q detJ_q B^T D(eta_q) B with D = diag(2eta,2eta,eta) in 2D and
 * diag(2eta,2eta,2eta,eta,eta,eta) in 3D (strain order xx,yy,zz,xy,xz,yz)
 * (L/Underworld/Rheology/src/ConstitutiveMatrixCartesian.cpp:238-429,
 *  ConstitutiveMatrix.c:206-211).  Ke is (dim*nen)^2 row-major. */
void uwo_element_K(const uwo_mesh* m, const double* ax0, const double* ax1, const double* ax2,
                   int64_t el, int nq, const double* xi, const double* wt, const double* eta, double* Ke) {
    const double* ax[3] = {ax0, ax1, ax2};
    int64_t nodes[27];
    double N[27], GNx[3][27];
    int dim = m->dim, nen = uwo_el_nodes(m), nd = dim * nen;
    uwo_element_nodes(m, el, nodes);
    memset(Ke, 0, sizeof(double) * nd * nd);
    for (int q = 0; q < nq; q++) {
        double detJ = global_derivs(m, ax, nodes, xi + q * dim, N, GNx);
        double f = detJ * wt[q], e = eta[q];
        for (int a = 0; a < nen; a++)
            for (int b = 0; b < nen; b++) {
                double ax_ = GNx[0][a], ay = GNx[1][a], bx = GNx[0][b], by = GNx[1][b];
                if (dim == 2) {
                    Ke[(a * 2 + 0) * nd + b * 2 + 0] += f * e * (2.0 * ax_ * bx + ay * by);
                    Ke[(a * 2 + 0) * nd + b * 2 + 1] += f * e * (ay * bx);
                    Ke[(a * 2 + 1) * nd + b * 2 + 0] += f * e * (ax_ * by);
                    Ke[(a * 2 + 1) * nd + b * 2 + 1] += f * e * (2.0 * ay * by + ax_ * bx);
                } else {
                    double az = GNx[2][a], bz = GNx[2][b];
                    double* r0 = Ke + (a * 3 + 0) * nd + b * 3;
                    double* r1 = Ke + (a * 3 + 1) * nd + b * 3;
                    double* r2 = Ke + (a * 3 + 2) * nd + b * 3;
                    r0[0] += f * e * (2.0 * ax_ * bx + ay * by + az * bz);
                    r0[1] += f * e * (ay * bx);
                    r0[2] += f * e * (az * bx);
                    r1[0] += f * e * (ax_ * by);
                    r1[1] += f * e * (2.0 * ay * by + ax_ * bx + az * bz);
                    r1[2] += f * e * (az * by);
                    r2[0] += f * e * (ax_ * bz);
                    r2[1] += f * e * (ay * bz);
                    r2[2] += f * e * (2.0 * az * bz + ax_ * bx + ay * by);
                }
            }
    }
}

/* G_e[A*dim+i][B] = sum_q w (-detJ) GNx[i][A] M_B(xi)
 * (L/StgFEM/Assembly/src/GradientStiffnessMatrixTerm.c:189-218). */
void uwo_element_G(const uwo_mesh* m, const double* ax0, const double* ax1, const double* ax2,
                   int porder, int64_t el, int nq, const double* xi, const double* wt, double* Ge) {
    const double* ax[3] = {ax0, ax1, ax2};
    int64_t nodes[27];
    double N[27], GNx[3][27], M[4];
    int dim = m->dim, nen = uwo_el_nodes(m), npn = uwo_pressure_nodes(dim, porder);
    uwo_element_nodes(m, el, nodes);
    memset(Ge, 0, sizeof(double) * dim * nen * npn);
    for (int q = 0; q < nq; q++) {
        double detJ = global_derivs(m, ax, nodes, xi + q * dim, N, GNx);
        uwo_pressure_shape(dim, porder, xi + q * dim, M);
        for (int a = 0; a < nen; a++)
            for (int i = 0; i < dim; i++)
                for (int b = 0; b < npn; b++)
                    Ge[(a * dim + i) * npn + b] += wt[q] * (-detJ) * (GNx[i][a] * M[b]);
    }
}

/* f_e[A*dim+i] = sum_q detJ w f_i(q) N_A
 * (L/Underworld/Utils/src/VectorAssemblyTerm_NA__Fn.cpp:143-202). */
void uwo_element_f(const uwo_mesh* m, const double* ax0, const double* ax1, const double* ax2,
                   int64_t el, int nq, const double* xi, const double* wt, const double* fq, double* fe) {
    const double* ax[3] = {ax0, ax1, ax2};
    int64_t nodes[27];
    double N[27], GNx[3][27];
    int dim = m->dim, nen = uwo_el_nodes(m);
    uwo_element_nodes(m, el, nodes);
    memset(fe, 0, sizeof(double) * dim * nen);
    for (int q = 0; q < nq; q++) {
        double detJ = global_derivs(m, ax, nodes, xi + q * dim, N, GNx);
        double factor = detJ * wt[q];
        for (int a = 0; a < nen; a++)
            for (int i = 0; i < dim; i++) fe[a * dim + i] += factor * fq[q * dim + i] * N[a];
    }
}

/* M_e[A][B] = sum_q w detJ F N_A N_B over the pressure basis
 * (L/Underworld/Utils/src/MatrixAssemblyTerm_NA__NB__Fn.cpp:129-190). */
void uwo_element_M(const uwo_mesh* m, const double* ax0, const double* ax1, const double* ax2,
                   int porder, int64_t el, int nq, const double* xi, const double* wt, const double* Fq,
                   double* Me) {
    const double* ax[3] = {ax0, ax1, ax2};
    int64_t nodes[27];
    double N[27], GNx[3][27], M[4];
    int dim = m->dim, npn = uwo_pressure_nodes(dim, porder);
    uwo_element_nodes(m, el, nodes);
    memset(Me, 0, sizeof(double) * npn * npn);
    for (int q = 0; q < nq; q++) {
        double detJ = global_derivs(m, ax, nodes, xi + q * dim, N, GNx);
        uwo_pressure_shape(dim, porder, xi + q * dim, M);
        for (int a = 0; a < npn; a++)
            for (int b = 0; b < npn; b++) Me[a * npn + b] += wt[q] * detJ * Fq[q] * M[a] * M[b];
    }
}

/* h_e[B] = sum_q w detJ F N_B over the pressure basis: the continuity source term
 * (VectorAssemblyTerm_NA__Fn on the pressure vector,
 * L/Underworld/Utils/src/VectorAssemblyTerm_NA__Fn.cpp:143-202; detJ from the velocity
 * geometry; added for fn_source at P/systems/_stokes.py:284-288). */
void uwo_element_h(const uwo_mesh* m, const double* ax0, const double* ax1, const double* ax2,
                   int porder, int64_t el, int nq, const double* xi, const double* wt, const double* Fq,
                   double* he) {
    const double* ax[3] = {ax0, ax1, ax2};
    int64_t nodes[27];
    double N[27], GNx[3][27], M[4];
    int dim = m->dim, npn = uwo_pressure_nodes(dim, porder);
    uwo_element_nodes(m, el, nodes);
    memset(he, 0, sizeof(double) * npn);
    for (int q = 0; q < nq; q++) {
        double detJ = global_derivs(m, ax, nodes, xi + q * dim, N, GNx);
        uwo_pressure_shape(dim, porder, xi + q * dim, M);
        double factor = detJ * wt[q];
        for (int b = 0; b < npn; b++) he[b] += factor * Fq[q] * M[b];
    }
}

/* S_e = G_e^T diag(K_e)^-1 G_e
 * (L/StgFEM/SLE/ProvidedSystems/StokesFlow/src/UzawaPreconditionerTerm.c:124-207). */
void uwo_element_S(int nv, int npn, const double* Ke, const double* Ge, double* Se) {
    memset(Se, 0, sizeof(double) * npn * npn);
    for (int r = 0; r < npn; r++)
        for (int c = 0; c < npn; c++)
            for (int v = 0; v < nv; v++)
                Se[r * npn + c] += Ge[v * npn + c] * (Ge[v * npn + r] / Ke[v * nv + v]);
}

/* ------------------------------------------------------------------------ */
/* Velocity interpolation and RK2 advection                                  */
/* ------------------------------------------------------------------------ */
/* FieldVariable_InterpolateValueAt on a regular mesh: search, Newton local
 * coordinates, node-order accumulation (L/StgFEM/Discretisation/src/
 * FeVariable.c:389-403,549-599,1007-1044).  vel is node-major [node][dim].
 * Returns 0 when the point is outside the mesh. */
int uwo_interpolate(const uwo_mesh* m, const double* ax0, const double* ax1, const double* ax2,
                    const double* vel, const double* x, double* v) {
    int64_t el, nodes[27];
    double xi[3], N[27];
    int dim = m->dim, nen = uwo_el_nodes(m);
    if (!uwo_search_element(m, x, &el)) return 0;
    uwo_global_to_local(m, ax0, ax1, ax2, el, x, xi);
    uwo_element_nodes(m, el, nodes);
    uwo_shape(dim, m->order, xi, N, NULL);
    for (int d = 0; d < dim; d++) v[d] = 0.0;
    for (int n = 0; n < nen; n++)
        for (int d = 0; d < dim; d++) v[d] += vel[nodes[n] * dim + d] * N[n];
    if (isinf(v[0]) || isinf(v[1]) || (dim == 3 && isinf(v[2]))) return 0;
    return 1;
}

/* TimeIntegrand_SecondOrder with first-order fallback
 * (L/StgDomain/Utils/src/TimeIntegrand.c:249-319,441-468) driven by
 * _SwarmAdvector_TimeDeriv (L/PICellerator/MaterialPoints/src/SwarmAdvector.c:238-312).
 * counts[0] += particles whose predictor evaluation failed (an error in the
 * reference), counts[1] += particles that fell back to first order. */
void uwo_rk2(const uwo_mesh* m, const double* ax0, const double* ax1, const double* ax2,
             const double* vel, double dt, int64_t p0, int64_t p1, double* coords, int64_t* counts) {
    int dim = m->dim;
    int64_t failed = 0, fallback = 0;
#pragma omp parallel for schedule(static) reduction(+ : failed, fallback)
    for (int64_t p = p0; p < p1; p++) {
        double* x = coords + p * dim;
        double x0[3], v[3];
        for (int d = 0; d < dim; d++) x0[d] = x[d];
        if (!uwo_interpolate(m, ax0, ax1, ax2, vel, x, v)) { failed++; continue; }
        for (int d = 0; d < dim; d++) x[d] = x0[d] + 0.5 * dt * v[d];
        if (uwo_interpolate(m, ax0, ax1, ax2, vel, x, v)) {
            for (int d = 0; d < dim; d++) x[d] = x0[d] + dt * v[d];
        } else {
            fallback++;
            for (int d = 0; d < dim; d++) x[d] = x0[d];
            uwo_interpolate(m, ax0, ax1, ax2, vel, x, v);
            for (int d = 0; d < dim; d++) x[d] = x0[d] + dt * v[d];
        }
    }
    counts[0] += failed;
    counts[1] += fallback;
}

/* ------------------------------------------------------------------------ */
/* Semi-Lagrangian departure values (SLCN advection-diffusion)               */
/* ------------------------------------------------------------------------ */
/* PeriodicUpdate, non-periodic: clamp one coordinate to the domain
 * (L/StgFEM/Utils/src/SemiLagrangianIntegrator.c:382-393). */
static void slcn_clamp(const uwo_mesh* m, double* p, int d) {
    if (p[d] < m->minc[d]) { p[d] = m->minc[d]; return; }
    if (p[d] > m->maxc[d]) p[d] = m->maxc[d];
}

/* InterpLagrange (SemiLagrangianIntegrator.c:357-380), one dof. */
static double slcn_lagrange(double x, const double* c, const double* v) {
    double r = 0.0;
    for (int n = 0; n < 4; n++) {
        double f = 1.0;
        for (int o = 0; o < 4; o++) {
            if (o == n) continue;
            f *= (x - c[o]) / (c[n] - c[o]);
        }
        r += v[n] * f;
    }
    return r;
}

/* SemiLagrangianIntegrator_BuildStaticStencils (:534-598), one axis, serial. */
static int slcn_stencil_start(int i, int n) {
    int s = i > 0 ? i - 1 : i;
    s += 3;
    return s >= n ? s - 4 : s - 3;
}

/* SemiLagrangianIntegrator_SolveNew (:600-653) on a Q1 mesh: each node is
 * traced back over dt with IntegrateRungeKutta (:267-302, classical RK4, the
 * reference's INV6 = 0.166666666667, every stage clamped to the domain); if the
 * launch point is within 1e-6 * minsep of the node the node value is kept,
 * else BicubicInterpolatorNew (:395-505) evaluates the 4^dim Lagrange
 * interpolant on the static stencil of the element holding the launch point.
 * Returns -1 if an axis has fewer than 4 nodes (the reference aborts). */
int uwo_slcn_phistar(const uwo_mesh* m, const double* ax0, const double* ax1, const double* ax2,
                     const double* vel, const double* phi, double dt, double minsep, double* out) {
    const double* ax[3] = {ax0, ax1, ax2};
    int dim = m->dim;
    int64_t nx[3] = {1, 1, 1};
    for (int d = 0; d < dim; d++) {
        nx[d] = uwo_nodes_per_axis(m, d);
        if (nx[d] < 4) return -1;
    }
    int64_t nn = nx[0] * nx[1] * nx[2];
    const double INV6 = 0.166666666667;
    for (int64_t i = 0; i < nn; i++) {
        int64_t id[3] = {i % nx[0], (i / nx[0]) % nx[1], i / (nx[0] * nx[1])};
        double x0[3] = {0, 0, 0}, xp[3] = {0, 0, 0}, pos[3] = {0, 0, 0};
        double k[4][3] = {{0}};
        for (int d = 0; d < dim; d++) x0[d] = ax[d][id[d]];
        uwo_interpolate(m, ax0, ax1, ax2, vel, x0, k[0]);
        for (int d = 0; d < dim; d++) { xp[d] = x0[d] - 0.5 * dt * k[0][d]; slcn_clamp(m, xp, d); }
        uwo_interpolate(m, ax0, ax1, ax2, vel, xp, k[1]);
        for (int d = 0; d < dim; d++) { xp[d] = x0[d] - 0.5 * dt * k[1][d]; slcn_clamp(m, xp, d); }
        uwo_interpolate(m, ax0, ax1, ax2, vel, xp, k[2]);
        for (int d = 0; d < dim; d++) { xp[d] = x0[d] - dt * k[2][d]; slcn_clamp(m, xp, d); }
        uwo_interpolate(m, ax0, ax1, ax2, vel, xp, k[3]);
        for (int d = 0; d < dim; d++) {
            pos[d] = x0[d] - INV6 * dt * (k[0][d] + 2.0 * k[1][d] + 2.0 * k[2][d] + k[3][d]);
            slcn_clamp(m, pos, d);
        }
        /* SemiLagrangianIntegrator_PointsAreClose(pos, x0, dim, 0, 1e-6 minsep) (:507-532) */
        double disp[3] = {0, 0, 0}, dot = 0.0;
        for (int d = 0; d < dim; d++) disp[d] = pos[d] - x0[d];
        for (int d = dim - 1; d >= 0; d--) dot = dot + disp[d] * disp[d];
        int64_t el;
        if (sqrt(dot) < 1e-6 * minsep || !uwo_search_element(m, pos, &el)) {
            out[i] = phi[i];
            continue;
        }
        int64_t e[3] = {el % m->res[0], (el / m->res[0]) % m->res[1], el / ((int64_t)m->res[0] * m->res[1])};
        int64_t s[3] = {0, 0, 0};
        double c[3][4];
        for (int d = 0; d < dim; d++) {
            s[d] = slcn_stencil_start((int)e[d], (int)nx[d]);
            for (int a = 0; a < 4; a++) c[d][a] = ax[d][s[d] + a];
        }
        double ptsX[4], ptsY[4], ptsZ[4];
        if (dim == 2) {
            for (int yi = 0; yi < 4; yi++) {
                for (int xi = 0; xi < 4; xi++) ptsX[xi] = phi[(s[0] + xi) + (s[1] + yi) * nx[0]];
                ptsY[yi] = slcn_lagrange(pos[0], c[0], ptsX);
            }
            out[i] = slcn_lagrange(pos[1], c[1], ptsY);
        } else {
            for (int zi = 0; zi < 4; zi++) {
                for (int yi = 0; yi < 4; yi++) {
                    for (int xi = 0; xi < 4; xi++)
                        ptsX[xi] = phi[(s[0] + xi) + (s[1] + yi) * nx[0] + (s[2] + zi) * nx[0] * nx[1]];
                    ptsY[yi] = slcn_lagrange(pos[0], c[0], ptsX);
                }
                ptsZ[zi] = slcn_lagrange(pos[1], c[1], ptsY);
            }
            out[i] = slcn_lagrange(pos[2], c[2], ptsZ);
        }
    }
    return 0;
}

/* FeMesh_CoordLocalToGlobal (L/StgFEM/Discretisation/src/FeMesh.c:333-360). */
void uwo_local_to_global(const uwo_mesh* m, const double* ax0, const double* ax1, const double* ax2,
                         int64_t el, const double* xi, double* x) {
    const double* ax[3] = {ax0, ax1, ax2};
    local_to_global(m, ax, el, xi, x);
}
