// Element geometry shared by the particle kernels (compiled with -fmad=false
// so that every multiply and add rounds separately, in the reference's order).
//
//   L/ = src/underworld/libUnderworld/
#pragma once
#include "uwg_internal.cuh"

struct uwg_geom {
    int dim, order;
    int res[3];
    int nx[3];             // nodes per axis
    double minc[3], maxc[3];
    const double* ax[3];
};

// Shape functions and local derivatives -------------------------------------------
// Bilinear: L/StgFEM/Discretisation/src/BilinearElementType.c:179-211
// Trilinear: L/StgFEM/Discretisation/src/TrilinearElementType.c:215-274
// Biquadratic: L/StgFEM/Discretisation/src/Biquadratic.c:138-200
template <int DIM, int ORDER> struct Shape;

template <> struct Shape<2, 1> {
    static constexpr int NEN = 4;
    __device__ static void N(const double* l, double* n) {
        double xi = l[0], eta = l[1];
        n[0] = 0.25 * (1.0 - xi) * (1.0 - eta);
        n[1] = 0.25 * (1.0 + xi) * (1.0 - eta);
        n[2] = 0.25 * (1.0 - xi) * (1.0 + eta);
        n[3] = 0.25 * (1.0 + xi) * (1.0 + eta);
    }
    __device__ static void dN(const double* l, double (*g)[NEN]) {
        double xi = l[0], eta = l[1];
        g[0][0] = -(0.25 * (1.0 - eta));
        g[0][1] = 0.25 * (1.0 - eta);
        g[0][3] = 0.25 * (1.0 + eta);
        g[0][2] = -(0.25 * (1.0 + eta));
        g[1][0] = -(0.25 * (1.0 - xi));
        g[1][1] = -(0.25 * (1.0 + xi));
        g[1][3] = 0.25 * (1.0 + xi);
        g[1][2] = 0.25 * (1.0 - xi);
    }
};

template <> struct Shape<3, 1> {
    static constexpr int NEN = 8;
    __device__ static void N(const double* l, double* n) {
        double xi = l[0], eta = l[1], zeta = l[2];
        n[0] = 0.125 * (1.0 - xi) * (1.0 - eta) * (1.0 - zeta);
        n[2] = 0.125 * (1.0 - xi) * (1.0 + eta) * (1.0 - zeta);
        n[3] = 0.125 * (1.0 + xi) * (1.0 + eta) * (1.0 - zeta);
        n[1] = 0.125 * (1.0 + xi) * (1.0 - eta) * (1.0 - zeta);
        n[4] = 0.125 * (1.0 - xi) * (1.0 - eta) * (1.0 + zeta);
        n[6] = 0.125 * (1.0 - xi) * (1.0 + eta) * (1.0 + zeta);
        n[7] = 0.125 * (1.0 + xi) * (1.0 + eta) * (1.0 + zeta);
        n[5] = 0.125 * (1.0 + xi) * (1.0 - eta) * (1.0 + zeta);
    }
    __device__ static void dN(const double* l, double (*g)[NEN]) {
        double xi = l[0], eta = l[1], zeta = l[2];
        g[0][0] = -(0.125 * (1.0 - eta) * (1.0 - zeta));
        g[0][2] = -(0.125 * (1.0 + eta) * (1.0 - zeta));
        g[0][3] = 0.125 * (1.0 + eta) * (1.0 - zeta);
        g[0][1] = 0.125 * (1.0 - eta) * (1.0 - zeta);
        g[0][4] = -(0.125 * (1.0 - eta) * (1.0 + zeta));
        g[0][6] = -(0.125 * (1.0 + eta) * (1.0 + zeta));
        g[0][7] = 0.125 * (1.0 + eta) * (1.0 + zeta);
        g[0][5] = 0.125 * (1.0 - eta) * (1.0 + zeta);
        g[1][0] = -(0.125 * (1.0 - xi) * (1.0 - zeta));
        g[1][2] = 0.125 * (1.0 - xi) * (1.0 - zeta);
        g[1][3] = 0.125 * (1.0 + xi) * (1.0 - zeta);
        g[1][1] = -(0.125 * (1.0 + xi) * (1.0 - zeta));
        g[1][4] = -(0.125 * (1.0 - xi) * (1.0 + zeta));
        g[1][6] = 0.125 * (1.0 - xi) * (1.0 + zeta);
        g[1][7] = 0.125 * (1.0 + xi) * (1.0 + zeta);
        g[1][5] = -(0.125 * (1.0 + xi) * (1.0 + zeta));
        g[2][0] = -0.125 * (1.0 - xi) * (1.0 - eta);
        g[2][2] = -0.125 * (1.0 - xi) * (1.0 + eta);
        g[2][3] = -0.125 * (1.0 + xi) * (1.0 + eta);
        g[2][1] = -0.125 * (1.0 + xi) * (1.0 - eta);
        g[2][4] = 0.125 * (1.0 - xi) * (1.0 - eta);
        g[2][6] = 0.125 * (1.0 - xi) * (1.0 + eta);
        g[2][7] = 0.125 * (1.0 + xi) * (1.0 + eta);
        g[2][5] = 0.125 * (1.0 + xi) * (1.0 - eta);
    }
};

template <> struct Shape<2, 2> {
    static constexpr int NEN = 9;
    __device__ static void N(const double* l, double* n) {
        double xi = l[0], eta = l[1];
        double a0 = xi - 1.0, b0 = eta - 1.0;
        double a1 = 1.0 - xi * xi, b1 = 1.0 - eta * eta;
        double a2 = xi + 1.0, b2 = eta + 1.0;
        double m0 = 0.5 * xi, m1 = 0.5 * eta, m2 = 0.25 * xi * eta;
        n[0] = m2 * a0 * b0; n[1] = m1 * a1 * b0; n[2] = m2 * a2 * b0;
        n[3] = m0 * a0 * b1; n[4] = a1 * b1;      n[5] = m0 * a2 * b1;
        n[6] = m2 * a0 * b2; n[7] = m1 * a1 * b2; n[8] = m2 * a2 * b2;
    }
    __device__ static void dN(const double* l, double (*g)[NEN]) {
        double xi = l[0], eta = l[1];
        double a0 = xi - 1.0, b0 = eta - 1.0;
        double a1 = xi + 1.0, b1 = eta + 1.0;
        double a2 = 2.0 * xi - 1.0, b2 = 2.0 * eta - 1.0;
        double a3 = 2.0 * xi + 1.0, b3 = 2.0 * eta + 1.0;
        double a4 = 1.0 - xi * xi, b4 = 1.0 - eta * eta;
        double m0 = 0.25 * xi, m1 = 0.25 * eta, m2 = -xi * eta;
        g[0][0] = m1 * a2 * b0; g[0][2] = m1 * a3 * b0;
        g[0][6] = m1 * a2 * b1; g[0][8] = m1 * a3 * b1;
        g[1][0] = m0 * a0 * b2; g[1][2] = m0 * a1 * b2;
        g[1][6] = m0 * a0 * b3; g[1][8] = m0 * a1 * b3;
        g[0][1] = m2 * b0; g[0][7] = m2 * b1;
        g[0][3] = 0.5 * a2 * b4; g[0][5] = 0.5 * a3 * b4;
        g[1][1] = 0.5 * a4 * b2; g[1][7] = 0.5 * a4 * b3;
        g[1][3] = m2 * a0; g[1][5] = m2 * a1;
        g[0][4] = -2.0 * xi * b4;
        g[1][4] = -2.0 * eta * a4;
    }
};

// Triquadratic: L/StgFEM/Discretisation/src/Triquadratic.c:193-400.  Node n =
// a + 3b + 9c (x fastest); basis = m * A_a * B_b * C_c where A_0 = xi - 1,
// A_1 = 1 - xi^2, A_2 = xi + 1 (B, C likewise) and m is the product of the
// 1/2-scaled coordinates of the axes on which the node is a corner node
// (m0..m6 of the reference); derivatives replace one factor by its derivative
// (xi - 1/2, -2 xi, xi + 1/2) and keep the other axes' m factor.  Same products
// in the same order as the reference.
template <> struct Shape<3, 2> {
    static constexpr int NEN = 27;
    __device__ static void N(const double* l, double* n) {
        const double xi = l[0], eta = l[1], zeta = l[2];
        const double A[3] = {xi - 1.0, 1.0 - xi * xi, xi + 1.0};
        const double B[3] = {eta - 1.0, 1.0 - eta * eta, eta + 1.0};
        const double C[3] = {zeta - 1.0, 1.0 - zeta * zeta, zeta + 1.0};
        const double m0 = 0.5 * xi, m1 = 0.5 * eta, m2 = 0.5 * zeta;
        const double m3 = 0.25 * xi * eta, m4 = 0.25 * xi * zeta, m5 = 0.25 * eta * zeta;
        const double m6 = 0.125 * xi * eta * zeta;
#pragma unroll
        for (int k = 0; k < 27; k++) {
            const int a = k % 3, b = (k / 3) % 3, c = k / 9;
            const bool ex = a != 1, ey = b != 1, ez = c != 1;
            const int sel = (ex ? 4 : 0) | (ey ? 2 : 0) | (ez ? 1 : 0);
            if (sel == 0) n[k] = A[a] * B[b] * C[c];
            else {
                const double m = sel == 7 ? m6 : sel == 3 ? m5 : sel == 5 ? m4 : sel == 6 ? m3
                               : sel == 1 ? m2 : sel == 2 ? m1 : m0;
                n[k] = m * A[a] * B[b] * C[c];
            }
        }
    }
    __device__ static void dN(const double* l, double (*g)[NEN]) {
        const double xi = l[0], eta = l[1], zeta = l[2];
        const double A[3] = {xi - 1.0, 1.0 - xi * xi, xi + 1.0};
        const double B[3] = {eta - 1.0, 1.0 - eta * eta, eta + 1.0};
        const double C[3] = {zeta - 1.0, 1.0 - zeta * zeta, zeta + 1.0};
        const double dA[3] = {xi - 0.5, -2.0 * xi, xi + 0.5};
        const double dB[3] = {eta - 0.5, -2.0 * eta, eta + 0.5};
        const double dC[3] = {zeta - 0.5, -2.0 * zeta, zeta + 0.5};
        const double m0 = 0.5 * xi, m1 = 0.5 * eta, m2 = 0.5 * zeta;
        const double m3 = 0.25 * xi * eta, m4 = 0.25 * xi * zeta, m5 = 0.25 * eta * zeta;
#pragma unroll
        for (int k = 0; k < 27; k++) {
            const int a = k % 3, b = (k / 3) % 3, c = k / 9;
            const bool ex = a != 1, ey = b != 1, ez = c != 1;
            // d/dxi: m over (y, z); d/deta: m over (x, z); d/dzeta: m over (x, y)
            if (ey && ez) g[0][k] = dA[a] * m5 * B[b] * C[c];
            else if (ey) g[0][k] = dA[a] * m1 * B[b] * C[c];
            else if (ez) g[0][k] = dA[a] * m2 * B[b] * C[c];
            else g[0][k] = dA[a] * B[b] * C[c];
            if (ex && ez) g[1][k] = dB[b] * m4 * A[a] * C[c];
            else if (ex) g[1][k] = dB[b] * m0 * A[a] * C[c];
            else if (ez) g[1][k] = dB[b] * m2 * A[a] * C[c];
            else g[1][k] = dB[b] * A[a] * C[c];
            if (ex && ey) g[2][k] = dC[c] * m3 * A[a] * B[b];
            else if (ex) g[2][k] = dC[c] * m0 * A[a] * B[b];
            else if (ey) g[2][k] = dC[c] * m1 * A[a] * B[b];
            else g[2][k] = dC[c] * A[a] * B[b];
        }
    }
};

// Element node coordinate (local node n, axis d) of element (ex,ey,ez), x fastest.
template <int DIM, int ORDER>
__device__ __forceinline__ double node_coord(const uwg_geom& g, const int* eidx, int n, int d) {
    constexpr int K = ORDER + 1;
    int li = d == 0 ? n % K : (d == 1 ? (n / K) % K : n / (K * K));
    return g.ax[d][eidx[d] * ORDER + li];
}

// Mesh_RegularAlgorithms_SearchElements (L/StgDomain/Mesh/src/Mesh_RegularAlgorithms.c:174-205)
// with sep = (max - min) / res (:154).  Writes per-axis element indices.
template <int DIM>
__device__ bool search_element(const uwg_geom& g, const double* p, int* inds) {
#pragma unroll
    for (int d = 0; d < DIM; d++) {
        double sep = (g.maxc[d] - g.minc[d]) / g.res[d];
        if (uwg_num_approx(p[d] - g.maxc[d], 0.0)) inds[d] = g.res[d] - 1;
        else if (p[d] < g.minc[d] || p[d] > g.maxc[d]) return false;
        else {
            double out = (p[d] - g.minc[d]) / sep;
            double integer;
            double frac = modf(out, &integer);
            unsigned u = (unsigned)integer;
            if (u > 0 && uwg_num_approx(frac, 0.0)) u--;
            inds[d] = (int)u;
        }
    }
    return true;
}

// _ElementCellLayout_CellOf (L/StgDomain/Swarm/src/ElementCellLayout.c:291-320)
template <int DIM>
__device__ int64_t cell_of(const uwg_geom& g, const double* p, int64_t n_el) {
#pragma unroll
    for (int d = 0; d < DIM; d++)
        if (p[d] < g.minc[d] || p[d] > g.maxc[d]) return n_el;
    int inds[3] = {0, 0, 0};
    if (!search_element<DIM>(g, p, inds)) return n_el;
    return inds[0] + (int64_t)g.res[0] * (inds[1] + (int64_t)g.res[1] * inds[2]);
}

__device__ __forceinline__ void el_index(const uwg_geom& g, int64_t el, int* eidx) {
    eidx[0] = (int)(el % g.res[0]);
    eidx[1] = (int)((el / g.res[0]) % g.res[1]);
    eidx[2] = (int)(el / ((int64_t)g.res[0] * g.res[1]));
}

// TensorArray_SolveSystem (L/StgDomain/Geometry/src/TensorMath.c:959-1010)
template <int DIM>
__device__ __forceinline__ void solve_system(const double* t, double* s, const double* r) {
    if (DIM == 3) {
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

// Newton global -> local (L/StgFEM/Discretisation/src/ElementType.c:177-301):
// start at 0, stop when max |increment| < 1e-4, 100 iterations at most,
// failure sets xi[0] = 1.1.
template <int DIM, int ORDER>
__device__ void global_to_local(const uwg_geom& g, const int* eidx, const double* x, double* xi) {
    constexpr int NEN = Shape<DIM, ORDER>::NEN;
    double N[NEN], G[DIM][NEN];
#pragma unroll
    for (int d = 0; d < DIM; d++) xi[d] = 0.0;
    for (int it = 0; it < 100; it++) {
        double J[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0}, r[3] = {0, 0, 0}, dxi[3];
        Shape<DIM, ORDER>::N(xi, N);
        Shape<DIM, ORDER>::dN(xi, G);
#pragma unroll
        for (int n = 0; n < NEN; n++) {
            double vx = node_coord<DIM, ORDER>(g, eidx, n, 0);
            double vy = node_coord<DIM, ORDER>(g, eidx, n, 1);
            if (DIM == 2) {
                J[0] += G[0][n] * vx;
                J[1] += G[1][n] * vx;
                J[2] += G[0][n] * vy;
                J[3] += G[1][n] * vy;
                r[0] -= N[n] * vx;
                r[1] -= N[n] * vy;
            } else {
                double vz = node_coord<DIM, ORDER>(g, eidx, n, 2);
                J[0] += G[0][n] * vx;
                J[1] += G[1][n] * vx;
                J[3] += G[0][n] * vy;
                J[4] += G[1][n] * vy;
                r[0] -= N[n] * vx;
                r[1] -= N[n] * vy;
                J[2] += G[DIM - 1][n] * vx;
                J[5] += G[DIM - 1][n] * vy;
                J[6] += G[0][n] * vz;
                J[7] += G[1][n] * vz;
                J[8] += G[DIM - 1][n] * vz;
                r[2] -= N[n] * vz;
            }
        }
        r[0] += x[0];
        r[1] += x[1];
        if (DIM == 3) r[2] += x[2];
        solve_system<DIM>(J, dxi, r);
        xi[0] += dxi[0];
        xi[1] += dxi[1];
        if (DIM == 3) xi[2] += dxi[2];
        double mr = fabs(dxi[0]);
        if (mr < fabs(dxi[1])) mr = fabs(dxi[1]);
        if (DIM == 3 && mr < fabs(dxi[2])) mr = fabs(dxi[2]);
        if (mr < 0.0001) return;
    }
    xi[0] = 1.1;
}
