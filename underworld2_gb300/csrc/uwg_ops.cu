// Stokes operators on regular Q1/dQ0 meshes.
//
// Viscous operator.  On an affine (axis-aligned) element the PIC integrand of
// K_e = sum_q eta_q w_q detJ B^T D B (L/Underworld/Rheology/src/
// ConstitutiveMatrixCartesian.cpp:238-429) is, for every particle, a polynomial
// of degree <= 2 per axis in the local coordinate.  Lagrange interpolation on the
// 3-point tensor rule s in {-1, 0, 1} reproduces such polynomials exactly, so
//     W_j = sum_q eta_q w_q detJ_q l_j(xi_q)          (3^dim weights per element)
// gives K_e = sum_j W_j B(s_j)^T D B(s_j) identically (up to rounding): an exact,
// compact coefficient set that the matrix-free apply reads instead of K_e.
// The same identity coarsens W to the parent element of a twice-coarser mesh,
// which makes rediscretised coarse operators equal to Galerkin P^T K P.
//
// Gradient operator.  G_e[A,i] = -int_e dN_A/dx_i (dQ0 pressure, evaluated
// exactly; L/StgFEM/Assembly/src/GradientStiffnessMatrixTerm.c:129-219 uses
// Gauss quadrature, which is exact for this integrand).
//
// Schur preconditioner.  S_e = G_e^T diag(K_e)^-1 G_e - M_e
// (L/StgFEM/SLE/ProvidedSystems/StokesFlow/src/UzawaPreconditionerTerm.c:124-207):
// 1x1 per element for dQ0, so the assembled preconditioner is diagonal.
//
//   L/ = src/underworld/libUnderworld/
#include <algorithm>
#include <cmath>
#include <vector>

#include "uwg_ops.cuh"

static inline unsigned nblk(int64_t n, int t = 256) { return (unsigned)((n + t - 1) / t); }

uwg_lgeom uwg_level_geom(const uwg_ctx* c, int l) {
    uwg_lgeom g;
    const uwg_level& L = c->lev[l];
    g.dim = c->dim;
    g.order = L.order > 0 ? L.order : 1;
    for (int d = 0; d < 3; d++) {
        g.res[d] = L.res[d];
        g.nx[d] = d < c->dim ? L.res[d] * g.order + 1 : 1;
        g.ax[d] = L.ax[d];
    }
    g.n_el = L.n_el;
    g.n_nodes = L.n_nodes;
    return g;
}

__device__ __forceinline__ void q1_elem(const uwg_lgeom& g, int64_t e, int64_t* nodes, double* h) {
    int ex = (int)(e % g.res[0]);
    int ey = (int)((e / g.res[0]) % g.res[1]);
    int ez = g.dim == 3 ? (int)(e / ((int64_t)g.res[0] * g.res[1])) : 0;
    h[0] = g.ax[0][ex + 1] - g.ax[0][ex];
    h[1] = g.ax[1][ey + 1] - g.ax[1][ey];
    h[2] = g.dim == 3 ? g.ax[2][ez + 1] - g.ax[2][ez] : 1.0;
    int64_t nx = g.nx[0], ny = g.nx[1];
    int nn = g.dim == 3 ? 8 : 4;
    for (int n = 0; n < nn; n++) {
        int i = n & 1, j = (n >> 1) & 1, k = (n >> 2) & 1;
        nodes[n] = (ex + i) + nx * ((ey + j) + ny * (int64_t)(ez + k));
    }
}

// 1D quadratic Lagrange basis on {-1, 0, 1}
__device__ __forceinline__ void lag3(double s, double* l) {
    l[0] = 0.5 * s * (s - 1.0);
    l[1] = 1.0 - s * s;
    l[2] = 0.5 * s * (s + 1.0);
}

// Q1 basis value N_n(xi) (product form; assembly parity is to a tolerance)
template <int DIM>
__device__ __forceinline__ void q1_basis(const double* xi, double* N) {
    for (int n = 0; n < (DIM == 3 ? 8 : 4); n++) {
        double v = 1.0;
        for (int d = 0; d < DIM; d++) {
            double sg = ((n >> d) & 1) ? 1.0 : -1.0;
            v *= 0.5 * (1.0 + sg * xi[d]);
        }
        N[n] = v;
    }
}

// ---------------------------------------------------------------------------
// Assembly from the PIC integration points: one thread per element.
//   W[j*n_el + e] = sum_q eta w detJ l_j(xi_q)
//   f[node*dim + i] += sum_q w detJ body_i N_A(xi_q)        (atomic scatter)
//   Mp[e] = sum_q w detJ (-1/lambda_q)                         (optional)
// ---------------------------------------------------------------------------
template <int DIM>
__global__ void k_assemble_q1(uwg_lgeom g, const int32_t* off, const int32_t* list, const double* ip_xi,
                              const double* ip_w, const double* eta_p, const double* body_p,
                              const double* lambda_p, double* W, double* f, double* Mp) {
    constexpr int NQ = DIM == 3 ? 27 : 9;
    constexpr int NEN = DIM == 3 ? 8 : 4;
    int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (e >= g.n_el) return;
    int64_t nodes[8];
    double h[3];
    q1_elem(g, e, nodes, h);
    double detJ = DIM == 3 ? (h[0] * 0.5) * (h[1] * 0.5) * (h[2] * 0.5) : (h[0] * 0.5) * (h[1] * 0.5);
    double Wl[NQ];
    double fe[NEN * DIM];
    double mp = 0.0;
    for (int j = 0; j < NQ; j++) Wl[j] = 0.0;
    for (int j = 0; j < NEN * DIM; j++) fe[j] = 0.0;
    int32_t s0 = off[e], s1 = off[e + 1];
    for (int32_t s = s0; s < s1; s++) {
        int32_t p = list[s];
        double xi[3];
        for (int d = 0; d < DIM; d++) xi[d] = ip_xi[(int64_t)s * DIM + d];
        double wd = ip_w[s] * detJ;
        double c = eta_p[p] * wd;
        double lx[3], ly[3], lz[3] = {1.0, 0.0, 0.0};
        lag3(xi[0], lx);
        lag3(xi[1], ly);
        if (DIM == 3) lag3(xi[DIM - 1], lz);
#pragma unroll
        for (int kz = 0; kz < (DIM == 3 ? 3 : 1); kz++)
#pragma unroll
            for (int ky = 0; ky < 3; ky++)
#pragma unroll
                for (int kx = 0; kx < 3; kx++) Wl[kx + 3 * ky + 9 * kz] += c * lx[kx] * ly[ky] * lz[kz];
        if (body_p) {
            double N[NEN];
            q1_basis<DIM>(xi, N);
#pragma unroll
            for (int a = 0; a < NEN; a++)
#pragma unroll
                for (int i = 0; i < DIM; i++) fe[a * DIM + i] += wd * body_p[(int64_t)p * DIM + i] * N[a];
        }
        if (lambda_p) mp += wd * -lambda_p[p];
    }
    for (int j = 0; j < NQ; j++) W[(int64_t)j * g.n_el + e] = Wl[j];
    if (body_p)
        for (int a = 0; a < NEN; a++)
            for (int i = 0; i < DIM; i++) atomicAdd(&f[nodes[a] * DIM + i], fe[a * DIM + i]);
    if (Mp) Mp[e] = mp;
}

// ---------------------------------------------------------------------------
// Local derivative dN_n/dxi_d at the 3-point rule position (pa,pb,pc), Q1.
// ---------------------------------------------------------------------------
template <int DIM>
__device__ __forceinline__ double q1_lderiv(int n, int d, const int* pt) {
    // (1 + sg s)/2 at s = -1, 0, 1 : sg=-1 -> 1, .5, 0 ; sg=+1 -> 0, .5, 1
    double v = 1.0;
    for (int e = 0; e < DIM; e++) {
        int sgp = (n >> e) & 1;
        if (e == d) v *= sgp ? 0.5 : -0.5;
        else v *= (pt[e] == 1) ? 0.5 : ((pt[e] == 2) == (sgp == 1) ? 1.0 : 0.0);
    }
    return v;
}

// Element diagonal of K_e from W (and, on the finest level, the Schur block).
template <int DIM>
__global__ void k_diag_q1(uwg_lgeom g, const double* W, const uint8_t* bc, double* diag, double* shat,
                          const double* Mp) {
    constexpr int NQ = DIM == 3 ? 27 : 9;
    constexpr int NEN = DIM == 3 ? 8 : 4;
    int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (e >= g.n_el) return;
    int64_t nodes[8];
    double h[3];
    q1_elem(g, e, nodes, h);
    double hi[3] = {2.0 / h[0], 2.0 / h[1], 2.0 / h[2]};
    double kd[NEN * DIM];
    for (int v = 0; v < NEN * DIM; v++) kd[v] = 0.0;
    for (int j = 0; j < NQ; j++) {
        int pt[3] = {j % 3, (j / 3) % 3, DIM == 3 ? j / 9 : 1};
        double w = W[(int64_t)j * g.n_el + e];
        for (int n = 0; n < NEN; n++) {
            double gx[3];
            for (int d = 0; d < DIM; d++) gx[d] = hi[d] * q1_lderiv<DIM>(n, d, pt);
            double s2 = 0.0;
            for (int d = 0; d < DIM; d++) s2 += gx[d] * gx[d];
            for (int c = 0; c < DIM; c++) kd[n * DIM + c] += w * (s2 + gx[c] * gx[c]);
        }
    }
    for (int n = 0; n < NEN; n++)
        for (int c = 0; c < DIM; c++) {
            int64_t dof = nodes[n] * DIM + c;
            if (!bc[dof]) atomicAdd(&diag[dof], kd[n * DIM + c]);
        }
    if (shat) {
        // G_e[A,i] = -sg_i(A) * prod_{d != i} h_d / 2^(dim-1)
        double s = 0.0;
        for (int n = 0; n < NEN; n++)
            for (int i = 0; i < DIM; i++) {
                double ge = 1.0;
                for (int d = 0; d < DIM; d++)
                    if (d != i) ge *= 0.5 * h[d];
                ge *= ((n >> i) & 1) ? -1.0 : 1.0;
                s += ge * (ge / kd[n * DIM + i]);
            }
        if (Mp) s -= Mp[e];
        shat[e] = s;
    }
}

__global__ void k_diag_bc(int64_t n, const uint8_t* bc, double* diag, float* diag32, double* inv) {
    int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    double d = bc[i] ? 1.0 : diag[i];
    diag[i] = d;
    diag32[i] = (float)d;
}

// ---------------------------------------------------------------------------
// Matrix-free K apply, sum-factorised on the 3-point rule.
// y = P K P x + (I - P) x with P zeroing Dirichlet dofs.
// ---------------------------------------------------------------------------
// Double-float numbers: value = hi + lo with |lo| <= ulp(hi) / 2, about 48
// significant bits from FP32 operations (Dekker's TwoProd through fmaf,
// Knuth's TwoSum; the intrinsics keep the compiler from contracting them).
// The element arithmetic of the FP64 refinement residual runs in it on the
// FP32 pipe, which on this GPU issues far more than the FP64 one.
struct dfl {
    float hi, lo;
    __device__ __forceinline__ dfl() {}
    __device__ __forceinline__ dfl(double v) : hi((float)v), lo((float)(v - (double)(float)v)) {}
    __device__ __forceinline__ dfl(float h, float l) : hi(h), lo(l) {}
};
__device__ __forceinline__ dfl operator+(dfl a, dfl b) {
    const float s = __fadd_rn(a.hi, b.hi);
    const float bb = __fsub_rn(s, a.hi);
    const float err = __fadd_rn(__fsub_rn(a.hi, __fsub_rn(s, bb)), __fsub_rn(b.hi, bb));
    const float t = __fadd_rn(err, __fadd_rn(a.lo, b.lo));
    const float h = __fadd_rn(s, t);
    return dfl(h, __fsub_rn(t, __fsub_rn(h, s)));
}
__device__ __forceinline__ dfl operator-(dfl a) { return dfl(-a.hi, -a.lo); }
__device__ __forceinline__ dfl operator-(dfl a, dfl b) { return a + (-b); }
__device__ __forceinline__ dfl operator*(dfl a, dfl b) {
    const float p = __fmul_rn(a.hi, b.hi);
    float e = fmaf(a.hi, b.hi, -p);
    e = fmaf(a.hi, b.lo, e);
    e = fmaf(a.lo, b.hi, e);
    const float h = __fadd_rn(p, e);
    return dfl(h, __fsub_rn(e, __fsub_rn(h, p)));
}
__device__ __forceinline__ dfl& operator+=(dfl& a, dfl b) { a = a + b; return a; }
__device__ __forceinline__ dfl& operator-=(dfl& a, dfl b) { a = a - b; return a; }

template <typename T>
__device__ __forceinline__ void up3(T a, T b, T* o) { o[0] = a; o[1] = (T)0.5 * (a + b); o[2] = b; }

template <typename T>
__global__ void k_bc_copy(int64_t n, const uint8_t* bc, const T* x, T* y) {
    int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i < n) y[i] = bc[i] ? x[i] : (T)0;
}

// y_e = K_e u_e for one 3D Q1 element from its equivalent-quadrature weights
// (sum-factorised on the 3-point rule).  hx,hy,hz = 2/h per axis.
template <typename T>
__device__ __forceinline__ void q1_3d_element(const T* __restrict__ Wp, int64_t stride, T hx, T hy, T hz,
                                              const T (&u)[8][3], T (&out)[8][3]) {
    // physical gradients on the 3x3 face grids
    T Gx[3][3][3], Gy[3][3][3], Gz[3][3][3];   // [c][p][q]
#pragma unroll
    for (int c = 0; c < 3; c++) {
        T a0[3], a1[3];
        // d/dx : depends on (y,z) point
        {
            T d00 = (T)0.5 * hx * (u[1][c] - u[0][c]), d10 = (T)0.5 * hx * (u[3][c] - u[2][c]);
            T d01 = (T)0.5 * hx * (u[5][c] - u[4][c]), d11 = (T)0.5 * hx * (u[7][c] - u[6][c]);
            up3(d00, d10, a0);
            up3(d01, d11, a1);
#pragma unroll
            for (int p = 0; p < 3; p++) up3(a0[p], a1[p], Gx[c][p]);   // Gx[c][py][pz]
        }
        {
            T d00 = (T)0.5 * hy * (u[2][c] - u[0][c]), d10 = (T)0.5 * hy * (u[3][c] - u[1][c]);
            T d01 = (T)0.5 * hy * (u[6][c] - u[4][c]), d11 = (T)0.5 * hy * (u[7][c] - u[5][c]);
            up3(d00, d10, a0);
            up3(d01, d11, a1);
#pragma unroll
            for (int p = 0; p < 3; p++) up3(a0[p], a1[p], Gy[c][p]);   // Gy[c][px][pz]
        }
        {
            T d00 = (T)0.5 * hz * (u[4][c] - u[0][c]), d10 = (T)0.5 * hz * (u[5][c] - u[1][c]);
            T d01 = (T)0.5 * hz * (u[6][c] - u[2][c]), d11 = (T)0.5 * hz * (u[7][c] - u[3][c]);
            up3(d00, d10, a0);
            up3(d01, d11, a1);
#pragma unroll
            for (int p = 0; p < 3; p++) up3(a0[p], a1[p], Gz[c][p]);   // Gz[c][px][py]
        }
    }
    // stresses summed along the derivative axis
    T Rx[3][3][3], Ry[3][3][3], Rz[3][3][3];
#pragma unroll
    for (int c = 0; c < 3; c++)
#pragma unroll
        for (int p = 0; p < 3; p++)
#pragma unroll
            for (int q = 0; q < 3; q++) { Rx[c][p][q] = 0; Ry[c][p][q] = 0; Rz[c][p][q] = 0; }
#pragma unroll
    for (int pz = 0; pz < 3; pz++)
#pragma unroll
        for (int py = 0; py < 3; py++)
#pragma unroll
            for (int px = 0; px < 3; px++) {
                T w = Wp[(int64_t)(px + 3 * py + 9 * pz) * stride];
                T uxx = Gx[0][py][pz], uxy = Gy[0][px][pz], uxz = Gz[0][px][py];
                T uyx = Gx[1][py][pz], uyy = Gy[1][px][pz], uyz = Gz[1][px][py];
                T uzx = Gx[2][py][pz], uzy = Gy[2][px][pz], uzz = Gz[2][px][py];
                T sxx = w * (uxx + uxx), syy = w * (uyy + uyy), szz = w * (uzz + uzz);
                T sxy = w * (uxy + uyx), sxz = w * (uxz + uzx), syz = w * (uyz + uzy);
                Rx[0][py][pz] += sxx; Ry[0][px][pz] += sxy; Rz[0][px][py] += sxz;
                Rx[1][py][pz] += sxy; Ry[1][px][pz] += syy; Rz[1][px][py] += syz;
                Rx[2][py][pz] += sxz; Ry[2][px][pz] += syz; Rz[2][px][py] += szz;
            }
    // transpose of the face interpolation and the derivative
#pragma unroll
    for (int c = 0; c < 3; c++) {
        // down-sample 3x3 -> 2x2: v[j][k] = sum L(j,p) L(k,q) R[p][q]
        T v[2][2];
#define DOWN(R_)                                                                          \
    {                                                                                     \
        T t0[3], t1[3];                                                                   \
        for (int q = 0; q < 3; q++) {                                                     \
            t0[q] = R_[c][0][q] + (T)0.5 * R_[c][1][q];                                   \
            t1[q] = R_[c][2][q] + (T)0.5 * R_[c][1][q];                                   \
        }                                                                                 \
        v[0][0] = t0[0] + (T)0.5 * t0[1]; v[0][1] = t0[2] + (T)0.5 * t0[1];               \
        v[1][0] = t1[0] + (T)0.5 * t1[1]; v[1][1] = t1[2] + (T)0.5 * t1[1];               \
    }
        DOWN(Rx);   // v[jy][kz]
        {
            T s = (T)0.5 * hx;
            out[0][c] = -s * v[0][0]; out[1][c] = s * v[0][0];
            out[2][c] = -s * v[1][0]; out[3][c] = s * v[1][0];
            out[4][c] = -s * v[0][1]; out[5][c] = s * v[0][1];
            out[6][c] = -s * v[1][1]; out[7][c] = s * v[1][1];
        }
        DOWN(Ry);   // v[ix][kz]
        {
            T s = (T)0.5 * hy;
            out[0][c] -= s * v[0][0]; out[2][c] += s * v[0][0];
            out[1][c] -= s * v[1][0]; out[3][c] += s * v[1][0];
            out[4][c] -= s * v[0][1]; out[6][c] += s * v[0][1];
            out[5][c] -= s * v[1][1]; out[7][c] += s * v[1][1];
        }
        DOWN(Rz);   // v[ix][jy]
        {
            T s = (T)0.5 * hz;
            out[0][c] -= s * v[0][0]; out[4][c] += s * v[0][0];
            out[1][c] -= s * v[1][0]; out[5][c] += s * v[1][0];
            out[2][c] -= s * v[0][1]; out[6][c] += s * v[0][1];
            out[3][c] -= s * v[1][1]; out[7][c] += s * v[1][1];
        }
#undef DOWN
    }
}

template <typename T>
__global__ void __launch_bounds__(128) k_applyK_q1_3d(uwg_lgeom g, const T* __restrict__ W,
                                                      const uint8_t* __restrict__ bc, bool mask_in,
                                                      const T* __restrict__ x, T* y) {
    int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (e >= g.n_el) return;
    int64_t nodes[8];
    double hd[3];
    q1_elem(g, e, nodes, hd);
    // 2/h in the operator's precision (an FP64 division costs dozens of FP64
    // instructions, and FP64 throughput is scarce on this GPU)
    const T hx = (T)2 / (T)hd[0], hy = (T)2 / (T)hd[1], hz = (T)2 / (T)hd[2];
    T u[8][3];
    bool fix[8][3];
#pragma unroll
    for (int n = 0; n < 8; n++)
#pragma unroll
        for (int c = 0; c < 3; c++) {
            int64_t dof = nodes[n] * 3 + c;
            fix[n][c] = bc[dof] != 0;
            u[n][c] = (fix[n][c] && mask_in) ? (T)0 : x[dof];
        }
    T out[8][3];
    q1_3d_element<T>(W + e, g.n_el, hx, hy, hz, u, out);
#pragma unroll
    for (int n = 0; n < 8; n++)
#pragma unroll
        for (int c = 0; c < 3; c++)
            if (!fix[n][c]) atomicAdd(&y[nodes[n] * 3 + c], out[n][c]);
}


// Tiled K apply (3D): a CTA owns an 8x8x4 tile of elements.
//  1. The tile's 9x9x5 nodal values are staged by cp.async row by row: one
//     warp per row of 27 contiguous values, so a lane's node index is fixed
//     and no per-slot integer division is left.  Dirichlet flags are staged
//     only for tiles that hold a Dirichlet dof (a per-tile flag, built with
//     the level); the other tiles never read the mask.
//  2. One thread per element adds K_e u_e into a shared tile (shared atomics).
//  3. Write-back, row by row: Dirichlet dofs y = x (the identity rows; every
//     tile holding the node writes the same value), nodes inside the tile a
//     plain store, nodes on the tile faces a global atomic add onto y, which
//     the caller zeroes first (a memset rather than a masked copy pass).
// Tiles without a Dirichlet dof take an element path without the mask.  Two
// persistent variants measured slower on the 128^3 workload: one double-
// buffering the next tile's copies behind the current tile's compute (0.272 ms
// against 0.1875 ms per apply), and one with the per-tile index tables hoisted
// out of the tile loop, element outputs in zero-haloed per-corner planes (a
// node's value = 8 shared loads without validity tests) and the next tile's
// copies behind the write-back (0.226 ms).  At 16 warps per SM the kernel is
// bound by instruction issue and latency, not by DRAM.
#define KT_X 8
#define KT_Y 8
#define KT_Z 4
#define KT_N (KT_X * KT_Y * KT_Z)

template <int BYTES>
__device__ __forceinline__ void cp_async_z(void* smem, const void* gmem, bool valid) {
    unsigned sa = (unsigned)__cvta_generic_to_shared(smem);
    if constexpr (BYTES == 16)
        asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(sa), "l"(gmem), "r"(valid ? 16 : 0));
    else
        asm volatile("cp.async.ca.shared.global [%0], [%1], %2, %3;\n" ::"r"(sa), "l"(gmem), "n"(BYTES),
                     "r"(valid ? BYTES : 0));
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory"); }

int64_t uwg_ops_ktiles(const int* res) {
    return (int64_t)((res[0] + KT_X - 1) / KT_X) * ((res[1] + KT_Y - 1) / KT_Y) * ((res[2] + KT_Z - 1) / KT_Z);
}

// Per-tile Dirichlet flag: 1 when any dof of the tile's nodes (halo included) is fixed.
__global__ void k_tile_bc_flags(uwg_lgeom g, const uint8_t* __restrict__ bc, uint8_t* __restrict__ flags) {
    constexpr int NX = KT_X + 1, NY = KT_Y + 1, NZ = KT_Z + 1, NN = NX * NY * NZ;
    int ntx = (g.res[0] + KT_X - 1) / KT_X, nty = (g.res[1] + KT_Y - 1) / KT_Y;
    int tile = blockIdx.x;
    int tx0 = (tile % ntx) * KT_X, ty0 = ((tile / ntx) % nty) * KT_Y, tz0 = (tile / (ntx * nty)) * KT_Z;
    int any = 0;
    for (int k = threadIdx.x; k < NN * 3; k += blockDim.x) {
        int nl = k / 3, c = k % 3;
        int gi = tx0 + nl % NX, gj = ty0 + (nl / NX) % NY, gk = tz0 + nl / (NX * NY);
        if (gi < g.nx[0] && gj < g.nx[1] && gk < g.nx[2])
            any |= bc[(gi + (int64_t)g.nx[0] * (gj + (int64_t)g.nx[1] * gk)) * 3 + c] != 0;
    }
    any = __syncthreads_or(any);
    if (threadIdx.x == 0) flags[tile] = (uint8_t)any;
}

constexpr int KT_NROW = (KT_Y + 1) * (KT_Z + 1), KT_ROW = 3 * (KT_X + 1);
constexpr int KT_NN3 = KT_NROW * KT_ROW;
constexpr int KT_NIT = (KT_NROW + KT_N / 32 - 1) / (KT_N / 32);
static_assert(KT_ROW <= 32, "one warp per staged row");

// Stage a tile's nodal values (cp.async) and, for a tile with a Dirichlet dof, its flags (plain loads).
template <typename T>
__device__ __forceinline__ void kt_stage_x(const uwg_lgeom& g, int tx0, int ty0, int tz0, const T* __restrict__ x,
                                           T* xs) {
    constexpr int NY = KT_Y + 1, NW = KT_N / 32;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, gi = tx0 + lane / 3;
    const int64_t gnx = g.nx[0], gny = g.nx[1];
#pragma unroll
    for (int it = 0; it < KT_NIT; it++) {
        const int r = warp + it * NW;
        if (r < KT_NROW && lane < KT_ROW) {
            const int gj = ty0 + r % NY, gk = tz0 + r / NY;
            const bool in = gi < g.nx[0] && gj < g.nx[1] && gk < g.nx[2];
            const int64_t dof = in ? (tx0 + gnx * (gj + gny * (int64_t)gk)) * 3 + lane : 0;
            cp_async_z<sizeof(T)>(&xs[r * KT_ROW + lane], x + dof, in);
        }
    }
}
__device__ __forceinline__ void kt_stage_bc(const uwg_lgeom& g, int tx0, int ty0, int tz0,
                                            const uint8_t* __restrict__ bc, uint8_t* bs) {
    constexpr int NY = KT_Y + 1, NW = KT_N / 32;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, gi = tx0 + lane / 3;
    const int64_t gnx = g.nx[0], gny = g.nx[1];
#pragma unroll
    for (int it = 0; it < KT_NIT; it++) {
        const int r = warp + it * NW;
        if (r < KT_NROW && lane < KT_ROW) {
            const int gj = ty0 + r % NY, gk = tz0 + r / NY;
            const bool in = gi < g.nx[0] && gj < g.nx[1] && gk < g.nx[2];
            bs[r * KT_ROW + lane] = in ? bc[(tx0 + gnx * (gj + gny * (int64_t)gk)) * 3 + lane] : (uint8_t)1;
        }
    }
}

// One element: gather u from the staged tile (Dirichlet dofs as zero when
// HAS_BC), K_e u_e, scatter into the shared accumulator (FP64), or return the
// 24 outputs for the gather write-back (FP32, out != nullptr).
template <typename T, bool HAS_BC>
__device__ __forceinline__ void kt_element(const T* xs, const uint8_t* bs, T* ys, const T* ws, int64_t wstride, T hx,
                                           T hy, T hz, T (*eo)[3] = nullptr) {
    constexpr int NX = KT_X + 1, NY = KT_Y + 1;
    const int li = threadIdx.x % KT_X, lj = (threadIdx.x / KT_X) % KT_Y, lk = threadIdx.x / (KT_X * KT_Y);
    T u[8][3], out[8][3];
#pragma unroll
    for (int n = 0; n < 8; n++) {
        const int sl = (li + (n & 1)) + NX * ((lj + ((n >> 1) & 1)) + NY * (lk + ((n >> 2) & 1)));
#pragma unroll
        for (int c = 0; c < 3; c++) u[n][c] = (HAS_BC && bs[sl * 3 + c]) ? (T)0 : xs[sl * 3 + c];
    }
    q1_3d_element<T>(ws, wstride, hx, hy, hz, u, out);
    if (eo) {
#pragma unroll
        for (int n = 0; n < 8; n++)
#pragma unroll
            for (int c = 0; c < 3; c++) eo[n][c] = out[n][c];
        return;
    }
#pragma unroll
    for (int n = 0; n < 8; n++) {
        const int sl = (li + (n & 1)) + NX * ((lj + ((n >> 1) & 1)) + NY * (lk + ((n >> 2) & 1)));
#pragma unroll
        for (int c = 0; c < 3; c++) atomicAdd(&ys[sl * 3 + c], out[n][c]);
    }
}

// Gather write-back (FP32): eo[(n * 3 + c) * KT_N + t] holds output (node n,
// component c) of the element of thread t (zero for elements outside the
// mesh); a node sums the outputs of the up to eight tile elements around it.
__device__ __forceinline__ void kt_writeback_gather(const uwg_lgeom& g, int tx0, int ty0, int tz0, bool has_bc,
                                                    const float* xs, const uint8_t* bs, const float* eo,
                                                    float* __restrict__ y) {
    constexpr int NY = KT_Y + 1, NW = KT_N / 32;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, ni = lane / 3, c = lane - 3 * (lane / 3), gi = tx0 + ni;
    const int64_t gnx = g.nx[0], gny = g.nx[1];
#pragma unroll
    for (int it = 0; it < KT_NIT; it++) {
        const int r = warp + it * NW;
        if (r < KT_NROW && lane < KT_ROW) {
            const int nj = r % NY, nk = r / NY;
            const int gj = ty0 + nj, gk = tz0 + nk;
            if (gi < g.nx[0] && gj < g.nx[1] && gk < g.nx[2]) {
                const int64_t dof = (tx0 + gnx * (gj + gny * (int64_t)gk)) * 3 + lane;
                const int k = r * KT_ROW + lane;
                if (has_bc && bs[k]) {
                    y[dof] = xs[k];
                } else {
                    // element (ni - dx, nj - dy, nk - dz) holds this node as its corner n = dx + 2 dy + 4 dz:
                    // one base address, constant offsets, validity from six per-axis tests
                    const bool x0 = ni < KT_X, x1 = ni > 0, y0 = nj < KT_Y, y1 = nj > 0, z0 = nk < KT_Z, z1 = nk > 0;
                    const float* b0 = eo + c * KT_N + ni + KT_X * (nj + KT_Y * nk);
                    float v = 0.f;
#pragma unroll
                    for (int n = 0; n < 8; n++) {
                        const int dx = n & 1, dy = (n >> 1) & 1, dz = n >> 2;
                        const bool ok = (dx ? x1 : x0) && (dy ? y1 : y0) && (dz ? z1 : z0);
                        if (ok) v += b0[n * 3 * KT_N - dx - KT_X * dy - KT_X * KT_Y * dz];
                    }
                    const bool interior = ni > 0 && ni < KT_X && nj > 0 && nj < KT_Y && nk > 0 && nk < KT_Z;
                    if (interior) y[dof] = v;
                    else atomicAdd(&y[dof], v);
                }
            }
        }
    }
}

// Write-back, row by row (see the comment above KT_X).
template <typename T>
__device__ __forceinline__ void kt_writeback(const uwg_lgeom& g, int tx0, int ty0, int tz0, bool has_bc, const T* xs,
                                             const uint8_t* bs, const T* ys, T* __restrict__ y) {
    constexpr int NY = KT_Y + 1, NW = KT_N / 32;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, ni = lane / 3, gi = tx0 + ni;
    const int64_t gnx = g.nx[0], gny = g.nx[1];
#pragma unroll
    for (int it = 0; it < KT_NIT; it++) {
        const int r = warp + it * NW;
        if (r < KT_NROW && lane < KT_ROW) {
            const int nj = r % NY, nk = r / NY;
            const int gj = ty0 + nj, gk = tz0 + nk;
            const int k = r * KT_ROW + lane;
            if (gi < g.nx[0] && gj < g.nx[1] && gk < g.nx[2]) {
                const int64_t dof = (tx0 + gnx * (gj + gny * (int64_t)gk)) * 3 + lane;
                if (has_bc && bs[k]) {
                    y[dof] = xs[k];
                } else {
                    const bool interior = ni > 0 && ni < KT_X && nj > 0 && nj < KT_Y && nk > 0 && nk < KT_Z;
                    if (interior) y[dof] = ys[k];
                    else atomicAdd(&y[dof], ys[k]);
                }
            }
        }
    }
}

// One CTA per tile.  FP32 (STAGE_W): the tile's 27 weight planes go to shared
// memory by cp.async (16-byte copies of 4-element rows when res_x % 4 == 0
// and n_el % 4 == 0), 2/h comes from the level's FP32 table, 2 CTAs per SM.
// FP64: weights straight from global memory, 2/h in FP64.
template <typename T, bool STAGE_W, bool VEC_W>
__global__ void __launch_bounds__(KT_N, STAGE_W ? 2 : 1) k_applyK_q1_3d_tiled(
    uwg_lgeom g, const T* __restrict__ W, const uint8_t* __restrict__ bc, const uint8_t* __restrict__ tile_bc,
    const float* __restrict__ h2x, const float* __restrict__ h2y, const float* __restrict__ h2z,
    const T* __restrict__ x, T* __restrict__ y) {
    __shared__ __align__(16) T xs[KT_NN3];
    __shared__ T ys[STAGE_W ? 1 : KT_NN3];
    __shared__ __align__(16) T ws[STAGE_W ? 27 * KT_N : 1];
    __shared__ uint8_t bs[KT_NN3];
    const int ntx = (g.res[0] + KT_X - 1) / KT_X, nty = (g.res[1] + KT_Y - 1) / KT_Y;
    const int tile = blockIdx.x;
    const int tx0 = (tile % ntx) * KT_X, ty0 = ((tile / ntx) % nty) * KT_Y, tz0 = (tile / (ntx * nty)) * KT_Z;
    const int li = threadIdx.x % KT_X, lj = (threadIdx.x / KT_X) % KT_Y, lk = threadIdx.x / (KT_X * KT_Y);
    const int ex = tx0 + li, ey = ty0 + lj, ez = tz0 + lk;
    const bool own = ex < g.res[0] && ey < g.res[1] && ez < g.res[2];
    const int64_t e = own ? ex + (int64_t)g.res[0] * (ey + (int64_t)g.res[1] * ez) : 0;
    if constexpr (STAGE_W) {
        if constexpr (VEC_W) {
            // 27 planes x 32 rows x 2 chunks of 16 bytes: thread t copies chunk (t & 63)
            // of planes t/64, t/64 + 4, ...: one address computation, then a stride of n_el
            static_assert(KT_X == 8 && KT_Y * KT_Z == 32 && KT_N == 256, "16-byte weight staging layout");
            const int q = threadIdx.x & 63, j0 = threadIdx.x >> 6, ch = q & 1, lyz = q >> 1;
            const int cx = tx0 + ch * 4, cy = ty0 + (lyz & (KT_Y - 1)), cz = tz0 + lyz / KT_Y;
            const bool in = cx < g.res[0] && cy < g.res[1] && cz < g.res[2];
            const float* src = (const float*)W + (in ? cx + (int64_t)g.res[0] * (cy + (int64_t)g.res[1] * cz) : 0) +
                               (int64_t)j0 * g.n_el;
            float* dst = (float*)ws + j0 * KT_N + KT_X * lyz + ch * 4;
            const int64_t step = 4 * g.n_el;
#pragma unroll
            for (int j = j0; j < 27; j += 4, src += step, dst += 4 * KT_N) cp_async_z<16>(dst, src, in);
        } else {
#pragma unroll
            for (int j = 0; j < 27; j++) cp_async_z<sizeof(T)>(&ws[j * KT_N + threadIdx.x], W + (int64_t)j * g.n_el + e, own);
        }
    }
    kt_stage_x<T>(g, tx0, ty0, tz0, x, xs);
    cp_async_commit();
    const bool has_bc = tile_bc[tile] != 0;
    if (has_bc) kt_stage_bc(g, tx0, ty0, tz0, bc, bs);
    if constexpr (!STAGE_W)
        for (int k = threadIdx.x; k < KT_NN3; k += KT_N) ys[k] = (T)0;
    T hx = (T)1, hy = (T)1, hz = (T)1;
    if (own) {
        if constexpr (STAGE_W) {
            hx = (T)__ldg(&h2x[ex]); hy = (T)__ldg(&h2y[ey]); hz = (T)__ldg(&h2z[ez]);
        } else {
            hx = (T)2 / (T)(g.ax[0][ex + 1] - g.ax[0][ex]);
            hy = (T)2 / (T)(g.ax[1][ey + 1] - g.ax[1][ey]);
            hz = (T)2 / (T)(g.ax[2][ez + 1] - g.ax[2][ez]);
        }
    }
    cp_async_wait<0>();
    __syncthreads();
    if constexpr (STAGE_W) {
        // outputs in registers, then (once every thread is done with the weights)
        // into the weight buffer for the gather write-back: no shared atomics
        T eo[8][3];
#pragma unroll
        for (int n = 0; n < 8; n++) eo[n][0] = eo[n][1] = eo[n][2] = (T)0;
        if (own) {
            if (has_bc) kt_element<T, true>(xs, bs, ys, ws + threadIdx.x, KT_N, hx, hy, hz, eo);
            else kt_element<T, false>(xs, bs, ys, ws + threadIdx.x, KT_N, hx, hy, hz, eo);
        }
        __syncthreads();
#pragma unroll
        for (int n = 0; n < 8; n++)
#pragma unroll
            for (int c = 0; c < 3; c++) ws[(n * 3 + c) * KT_N + threadIdx.x] = eo[n][c];
        __syncthreads();
        kt_writeback_gather(g, tx0, ty0, tz0, has_bc, (const float*)xs, bs, (const float*)ws, (float*)y);
    } else {
        if (own) {
            if (has_bc) kt_element<T, true>(xs, bs, ys, W + e, g.n_el, hx, hy, hz);
            else kt_element<T, false>(xs, bs, ys, W + e, g.n_el, hx, hy, hz);
        }
        __syncthreads();
        kt_writeback<T>(g, tx0, ty0, tz0, has_bc, xs, bs, ys, y);
    }
}

// The FP64 tiled apply (staging, Dirichlet rows, write-back as in
// k_applyK_q1_3d_tiled<double>) with the element arithmetic in double-float:
// nodal values converted on their way out of shared memory, W from its
// double-float copy, outputs accumulated in FP64.  For the refinement
// residual b - K x of the mixed-precision velocity solves.
__global__ void __launch_bounds__(KT_N, 1) k_applyK_q1_3d_tiled_df(uwg_lgeom g, const dfl* __restrict__ Wd,
                                                                   const uint8_t* __restrict__ bc,
                                                                   const uint8_t* __restrict__ tile_bc,
                                                                   const double* __restrict__ x, double* __restrict__ y) {
    __shared__ __align__(16) double xs[KT_NN3];
    __shared__ double ys[KT_NN3];
    __shared__ uint8_t bs[KT_NN3];
    constexpr int NX = KT_X + 1, NY = KT_Y + 1;
    const int ntx = (g.res[0] + KT_X - 1) / KT_X, nty = (g.res[1] + KT_Y - 1) / KT_Y;
    const int tile = blockIdx.x;
    const int tx0 = (tile % ntx) * KT_X, ty0 = ((tile / ntx) % nty) * KT_Y, tz0 = (tile / (ntx * nty)) * KT_Z;
    const int li = threadIdx.x % KT_X, lj = (threadIdx.x / KT_X) % KT_Y, lk = threadIdx.x / (KT_X * KT_Y);
    const int ex = tx0 + li, ey = ty0 + lj, ez = tz0 + lk;
    const bool own = ex < g.res[0] && ey < g.res[1] && ez < g.res[2];
    const int64_t e = own ? ex + (int64_t)g.res[0] * (ey + (int64_t)g.res[1] * ez) : 0;
    kt_stage_x<double>(g, tx0, ty0, tz0, x, xs);
    cp_async_commit();
    const bool has_bc = tile_bc[tile] != 0;
    if (has_bc) kt_stage_bc(g, tx0, ty0, tz0, bc, bs);
    for (int k = threadIdx.x; k < KT_NN3; k += KT_N) ys[k] = 0.0;
    dfl hx(1.0), hy(1.0), hz(1.0);
    if (own) {
        hx = dfl(2.0 / (g.ax[0][ex + 1] - g.ax[0][ex]));
        hy = dfl(2.0 / (g.ax[1][ey + 1] - g.ax[1][ey]));
        hz = dfl(2.0 / (g.ax[2][ez + 1] - g.ax[2][ez]));
    }
    cp_async_wait<0>();
    __syncthreads();
    if (own) {
        dfl u[8][3], out[8][3];
#pragma unroll
        for (int n = 0; n < 8; n++) {
            const int sl = (li + (n & 1)) + NX * ((lj + ((n >> 1) & 1)) + NY * (lk + ((n >> 2) & 1)));
#pragma unroll
            for (int c = 0; c < 3; c++) u[n][c] = (has_bc && bs[sl * 3 + c]) ? dfl(0.f, 0.f) : dfl(xs[sl * 3 + c]);
        }
        q1_3d_element<dfl>(Wd + e, g.n_el, hx, hy, hz, u, out);
#pragma unroll
        for (int n = 0; n < 8; n++) {
            const int sl = (li + (n & 1)) + NX * ((lj + ((n >> 1) & 1)) + NY * (lk + ((n >> 2) & 1)));
#pragma unroll
            for (int c = 0; c < 3; c++) atomicAdd(&ys[sl * 3 + c], (double)out[n][c].hi + (double)out[n][c].lo);
        }
    }
    __syncthreads();
    kt_writeback<double>(g, tx0, ty0, tz0, has_bc, xs, bs, ys, y);
}

__global__ void k_split_w_df(int64_t n, const double* __restrict__ w, float2* __restrict__ out) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i < n) {
        const float hi = (float)w[i];
        out[i] = make_float2(hi, (float)(w[i] - (double)hi));
    }
}

template <typename T>
__global__ void __launch_bounds__(128) k_applyK_q1_2d(uwg_lgeom g, const T* __restrict__ W,
                                                      const uint8_t* __restrict__ bc, bool mask_in,
                                                      const T* __restrict__ x, T* y) {
    int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (e >= g.n_el) return;
    int64_t nodes[8];
    double hd[3];
    q1_elem(g, e, nodes, hd);
    const T hx = (T)2 / (T)hd[0], hy = (T)2 / (T)hd[1];   // 2/h in the operator's precision
    T u[4][2];
    bool fix[4][2];
#pragma unroll
    for (int n = 0; n < 4; n++)
#pragma unroll
        for (int c = 0; c < 2; c++) {
            int64_t dof = nodes[n] * 2 + c;
            fix[n][c] = bc[dof] != 0;
            u[n][c] = (fix[n][c] && mask_in) ? (T)0 : x[dof];
        }
    T Gx[2][3], Gy[2][3];
#pragma unroll
    for (int c = 0; c < 2; c++) {
        up3((T)0.5 * hx * (u[1][c] - u[0][c]), (T)0.5 * hx * (u[3][c] - u[2][c]), Gx[c]);   // over py
        up3((T)0.5 * hy * (u[2][c] - u[0][c]), (T)0.5 * hy * (u[3][c] - u[1][c]), Gy[c]);   // over px
    }
    T Rx[2][3] = {{0, 0, 0}, {0, 0, 0}}, Ry[2][3] = {{0, 0, 0}, {0, 0, 0}};
#pragma unroll
    for (int py = 0; py < 3; py++)
#pragma unroll
        for (int px = 0; px < 3; px++) {
            T w = W[(int64_t)(px + 3 * py) * g.n_el + e];
            T uxx = Gx[0][py], uxy = Gy[0][px], uyx = Gx[1][py], uyy = Gy[1][px];
            T sxx = w * (uxx + uxx), syy = w * (uyy + uyy), sxy = w * (uxy + uyx);
            Rx[0][py] += sxx; Ry[0][px] += sxy;
            Rx[1][py] += sxy; Ry[1][px] += syy;
        }
    T out[4][2];
#pragma unroll
    for (int c = 0; c < 2; c++) {
        T v0 = Rx[c][0] + (T)0.5 * Rx[c][1], v1 = Rx[c][2] + (T)0.5 * Rx[c][1];   // over jy
        T s = (T)0.5 * hx;
        out[0][c] = -s * v0; out[1][c] = s * v0; out[2][c] = -s * v1; out[3][c] = s * v1;
        v0 = Ry[c][0] + (T)0.5 * Ry[c][1]; v1 = Ry[c][2] + (T)0.5 * Ry[c][1];       // over ix
        s = (T)0.5 * hy;
        out[0][c] -= s * v0; out[2][c] += s * v0; out[1][c] -= s * v1; out[3][c] += s * v1;
    }
#pragma unroll
    for (int n = 0; n < 4; n++)
#pragma unroll
        for (int c = 0; c < 2; c++)
            if (!fix[n][c]) atomicAdd(&y[nodes[n] * 2 + c], out[n][c]);
}

template <typename T>
int uwg_ops_applyK(uwg_ctx* c, int l, const T* x, T* y) {
    const uwg_level& L = c->lev[l];
    uwg_lgeom g = uwg_level_geom(c, l);
    const T* W;
    if constexpr (sizeof(T) == 8) W = (const T*)L.W64; else W = (const T*)L.W32;
    if (L.order == 1 && c->dim == 3 && L.tile_bc) {
        // y = 0, then the tiled kernel writes Dirichlet rows (y = x) and adds K x elsewhere
        UWG_CUDA(c, cudaMemsetAsync(y, 0, sizeof(T) * L.n_dof, c->stream));
        unsigned tiles = (unsigned)uwg_ops_ktiles(L.res);
        bool vec = (L.res[0] % 4) == 0 && (L.n_el % 4) == 0;
        if constexpr (sizeof(T) == 4) {
            if (vec)
                k_applyK_q1_3d_tiled<T, true, true><<<tiles, KT_N, 0, c->stream>>>(
                    g, W, L.bc, L.tile_bc, L.h2inv[0], L.h2inv[1], L.h2inv[2], x, y);
            else
                k_applyK_q1_3d_tiled<T, true, false><<<tiles, KT_N, 0, c->stream>>>(
                    g, W, L.bc, L.tile_bc, L.h2inv[0], L.h2inv[1], L.h2inv[2], x, y);
        } else {
            k_applyK_q1_3d_tiled<T, false, false><<<tiles, KT_N, 0, c->stream>>>(
                g, W, L.bc, L.tile_bc, nullptr, nullptr, nullptr, x, y);
        }
        UWG_CUDA(c, cudaGetLastError());
        return UWG_OK;
    }
    k_bc_copy<T><<<nblk(L.n_dof), 256, 0, c->stream>>>(L.n_dof, L.bc, x, y);
    if (L.order == 2) return uwg_q2_applyK<T>(c, x, y, true);
    if (c->dim == 3) {
        return uwg_set_error(c, UWG_ERR_STATE, "3D Q1 apply before the level's tile flags were built");
    } else {
        k_applyK_q1_2d<T><<<nblk(L.n_el, 128), 128, 0, c->stream>>>(g, W, L.bc, true, x, y);
    }
    UWG_CUDA(c, cudaGetLastError());
    return UWG_OK;
}

// y = P K x (Dirichlet dofs of x kept, rows of Dirichlet dofs zero): the
// lifting term K_fb g of the right-hand side.
int uwg_ops_applyK_lift(uwg_ctx* c, const double* x, double* y) {
    const uwg_level& L = c->lev[0];
    uwg_lgeom g = uwg_level_geom(c, 0);
    vk_zero<double>(c->stream, L.n_dof, y);
    if (L.order == 2) return uwg_q2_applyK<double>(c, x, y, false);
    if (c->dim == 3) k_applyK_q1_3d<double><<<nblk(L.n_el, 128), 128, 0, c->stream>>>(g, L.W64, L.bc, false, x, y);
    else k_applyK_q1_2d<double><<<nblk(L.n_el, 128), 128, 0, c->stream>>>(g, L.W64, L.bc, false, x, y);
    UWG_CUDA(c, cudaGetLastError());
    return UWG_OK;
}
int uwg_ops_applyK_refine(uwg_ctx* c, const double* x, double* y) {
    const uwg_level& L = c->lev[0];
    if (L.order == 2 && c->dim == 3 && c->q2_ke_df) {
        k_bc_copy<double><<<nblk(L.n_dof), 256, 0, c->stream>>>(L.n_dof, L.bc, x, y);
        return uwg_q2_3d_applyK_df(c, x, y);
    }
    if (L.order == 1 && c->dim == 3 && L.Wdf && L.tile_bc) {
        UWG_CUDA(c, cudaMemsetAsync(y, 0, sizeof(double) * L.n_dof, c->stream));
        k_applyK_q1_3d_tiled_df<<<(unsigned)uwg_ops_ktiles(L.res), KT_N, 0, c->stream>>>(
            uwg_level_geom(c, 0), reinterpret_cast<const dfl*>(L.Wdf), L.bc, L.tile_bc, x, y);
        UWG_CUDA(c, cudaGetLastError());
        return UWG_OK;
    }
    return uwg_ops_applyK<double>(c, 0, x, y);
}

template int uwg_ops_applyK<double>(uwg_ctx*, int, const double*, double*);
template int uwg_ops_applyK<float>(uwg_ctx*, int, const float*, float*);

// ---------------------------------------------------------------------------
// Gradient and divergence (dQ0), element-wise closed form of -int dN_A/dx_i.
// ---------------------------------------------------------------------------
template <int DIM>
__global__ void k_applyG(uwg_lgeom g, const uint8_t* bc, const double* p, double* y) {
    constexpr int NEN = DIM == 3 ? 8 : 4;
    int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (e >= g.n_el) return;
    int64_t nodes[8];
    double h[3];
    q1_elem(g, e, nodes, h);
    double pe = p[e];
    for (int n = 0; n < NEN; n++)
        for (int i = 0; i < DIM; i++) {
            int64_t dof = nodes[n] * DIM + i;
            if (bc[dof]) continue;
            double ge = 1.0;
            for (int d = 0; d < DIM; d++)
                if (d != i) ge *= 0.5 * h[d];
            ge *= ((n >> i) & 1) ? -1.0 : 1.0;
            atomicAdd(&y[dof], ge * pe);
        }
}

template <int DIM>
__global__ void k_applyGt(uwg_lgeom g, const uint8_t* bc, int only_bc, const double* u, double* q) {
    constexpr int NEN = DIM == 3 ? 8 : 4;
    int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (e >= g.n_el) return;
    int64_t nodes[8];
    double h[3];
    q1_elem(g, e, nodes, h);
    double s = 0.0;
    for (int n = 0; n < NEN; n++)
        for (int i = 0; i < DIM; i++) {
            int64_t dof = nodes[n] * DIM + i;
            if ((bc[dof] != 0) != (only_bc != 0)) continue;
            double ge = 1.0;
            for (int d = 0; d < DIM; d++)
                if (d != i) ge *= 0.5 * h[d];
            ge *= ((n >> i) & 1) ? -1.0 : 1.0;
            s += ge * u[dof];
        }
    q[e] = s;
}

// Node-centred (gather) gradient: v[n][c] = (G p)[n][c] / D[n][c] over the
// 2^dim cells around node n, Dirichlet dofs zero.  D may be null (no scaling).
// No atomics: every dof is written by one thread.
template <int DIM>
__global__ void k_gradG_nodes(uwg_lgeom g, const uint8_t* bc, const double* p, const double* D, double* v) {
    int64_t n = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (n >= g.n_nodes) return;
    int ni = (int)(n % g.nx[0]), nj = (int)((n / g.nx[0]) % g.nx[1]);
    int nk = DIM == 3 ? (int)(n / ((int64_t)g.nx[0] * g.nx[1])) : 0;
    double acc[3] = {0.0, 0.0, 0.0};
    for (int cz = 0; cz < (DIM == 3 ? 2 : 1); cz++)
        for (int cy = 0; cy < 2; cy++)
            for (int cx = 0; cx < 2; cx++) {
                int ex = ni - 1 + cx, ey = nj - 1 + cy, ez = DIM == 3 ? nk - 1 + cz : 0;
                if (ex < 0 || ex >= g.res[0] || ey < 0 || ey >= g.res[1] || (DIM == 3 && (ez < 0 || ez >= g.res[2])))
                    continue;
                double h[3] = {g.ax[0][ex + 1] - g.ax[0][ex], g.ax[1][ey + 1] - g.ax[1][ey],
                               DIM == 3 ? g.ax[2][ez + 1] - g.ax[2][ez] : 1.0};
                double pe = p[ex + (int64_t)g.res[0] * (ey + (int64_t)g.res[1] * ez)];
                int loc[3] = {1 - cx, 1 - cy, 1 - cz};   // node's local index in this cell
                for (int c = 0; c < DIM; c++) {
                    double ge = 1.0;
                    for (int d = 0; d < DIM; d++)
                        if (d != c) ge *= 0.5 * h[d];
                    acc[c] += (loc[c] ? -ge : ge) * pe;
                }
            }
    for (int c = 0; c < DIM; c++) {
        int64_t dof = n * DIM + c;
        v[dof] = bc[dof] ? 0.0 : (D ? acc[c] / D[dof] : acc[c]);
    }
}

// ---------------------------------------------------------------------------
// FP32 pressure-space operators of the weighted BFBt preconditioner (level l):
//   v = Dinv * (G p)  (node gather),  q = G^T v  (cell gather),
//   L p = G^T Dinv G p,  Dinv = 1/sqrt(diag K) on free dofs.
// ---------------------------------------------------------------------------
template <int DIM>
__global__ void k_gradG32(uwg_lgeom g, const uint8_t* bc, const float* p, const float* Dinv, float* v) {
    int64_t n = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (n >= g.n_nodes) return;
    int ni = (int)(n % g.nx[0]), nj = (int)((n / g.nx[0]) % g.nx[1]);
    int nk = DIM == 3 ? (int)(n / ((int64_t)g.nx[0] * g.nx[1])) : 0;
    float acc[3] = {0.f, 0.f, 0.f};
#pragma unroll
    for (int cz = 0; cz < (DIM == 3 ? 2 : 1); cz++)
#pragma unroll
        for (int cy = 0; cy < 2; cy++)
#pragma unroll
            for (int cx = 0; cx < 2; cx++) {
                int ex = ni - 1 + cx, ey = nj - 1 + cy, ez = DIM == 3 ? nk - 1 + cz : 0;
                if (ex < 0 || ex >= g.res[0] || ey < 0 || ey >= g.res[1] || (DIM == 3 && (ez < 0 || ez >= g.res[2])))
                    continue;
                float hx = (float)(g.ax[0][ex + 1] - g.ax[0][ex]), hy = (float)(g.ax[1][ey + 1] - g.ax[1][ey]);
                float hz = DIM == 3 ? (float)(g.ax[2][ez + 1] - g.ax[2][ez]) : 2.0f;
                float pe = p[ex + (int64_t)g.res[0] * (ey + (int64_t)g.res[1] * ez)];
                float a0 = 0.5f * hy * (DIM == 3 ? 0.5f * hz : 1.0f);
                float a1 = 0.5f * hx * (DIM == 3 ? 0.5f * hz : 1.0f);
                float a2 = 0.25f * hx * hy;
                acc[0] += (cx ? a0 : -a0) * pe;   // node local index 1 - cx along x
                acc[1] += (cy ? a1 : -a1) * pe;
                if (DIM == 3) acc[2] += (cz ? a2 : -a2) * pe;
            }
#pragma unroll
    for (int c = 0; c < DIM; c++) {
        int64_t dof = n * DIM + c;
        v[dof] = bc[dof] ? 0.f : (Dinv ? acc[c] * Dinv[dof] : acc[c]);
    }
}

template <int DIM>
__global__ void k_Gt32(uwg_lgeom g, const uint8_t* bc, const float* v, float* q) {
    int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (e >= g.n_el) return;
    int ex = (int)(e % g.res[0]), ey = (int)((e / g.res[0]) % g.res[1]);
    int ez = DIM == 3 ? (int)(e / ((int64_t)g.res[0] * g.res[1])) : 0;
    float hx = (float)(g.ax[0][ex + 1] - g.ax[0][ex]), hy = (float)(g.ax[1][ey + 1] - g.ax[1][ey]);
    float hz = DIM == 3 ? (float)(g.ax[2][ez + 1] - g.ax[2][ez]) : 2.0f;
    float a[3] = {0.5f * hy * (DIM == 3 ? 0.5f * hz : 1.0f), 0.5f * hx * (DIM == 3 ? 0.5f * hz : 1.0f), 0.25f * hx * hy};
    int64_t nx = g.nx[0], ny = g.nx[1];
    float s = 0.f;
#pragma unroll
    for (int n = 0; n < (DIM == 3 ? 8 : 4); n++) {
        int64_t node = (ex + (n & 1)) + nx * ((ey + ((n >> 1) & 1)) + ny * (int64_t)(ez + ((n >> 2) & 1)));
#pragma unroll
        for (int i = 0; i < DIM; i++) {
            int64_t dof = node * DIM + i;
            float ge = ((n >> i) & 1) ? -a[i] : a[i];
            s += bc[dof] ? 0.f : ge * v[dof];
        }
    }
    q[e] = s;
}

template <int DIM>
__global__ void k_Ldiag32(uwg_lgeom g, const uint8_t* bc, const float* Dinv, float* out) {
    int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (e >= g.n_el) return;
    int ex = (int)(e % g.res[0]), ey = (int)((e / g.res[0]) % g.res[1]);
    int ez = DIM == 3 ? (int)(e / ((int64_t)g.res[0] * g.res[1])) : 0;
    float hx = (float)(g.ax[0][ex + 1] - g.ax[0][ex]), hy = (float)(g.ax[1][ey + 1] - g.ax[1][ey]);
    float hz = DIM == 3 ? (float)(g.ax[2][ez + 1] - g.ax[2][ez]) : 2.0f;
    float a[3] = {0.5f * hy * (DIM == 3 ? 0.5f * hz : 1.0f), 0.5f * hx * (DIM == 3 ? 0.5f * hz : 1.0f), 0.25f * hx * hy};
    int64_t nx = g.nx[0], ny = g.nx[1];
    float s = 0.f;
    for (int n = 0; n < (DIM == 3 ? 8 : 4); n++) {
        int64_t node = (ex + (n & 1)) + nx * ((ey + ((n >> 1) & 1)) + ny * (int64_t)(ez + ((n >> 2) & 1)));
        for (int i = 0; i < DIM; i++) {
            int64_t dof = node * DIM + i;
            if (!bc[dof]) s += a[i] * a[i] * Dinv[dof];
        }
    }
    out[e] = s > 0.f ? s : 1.f;
}

__global__ void k_winv(int64_t n, const double* diag, const uint8_t* bc, float* out) {
    int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i < n) out[i] = bc[i] ? 0.f : (float)(1.0 / sqrt(diag[i]));
}

template <int DIM>
__global__ void k_cell_restrict32(uwg_lgeom gf, uwg_lgeom gc, const float* rf, float* rc) {
    int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (e >= gc.n_el) return;
    int ex = (int)(e % gc.res[0]), ey = (int)((e / gc.res[0]) % gc.res[1]);
    int ez = DIM == 3 ? (int)(e / ((int64_t)gc.res[0] * gc.res[1])) : 0;
    float s = 0.f;
    for (int cz = 0; cz < (DIM == 3 ? 2 : 1); cz++)
        for (int cy = 0; cy < 2; cy++)
            for (int cx = 0; cx < 2; cx++)
                s += rf[(2 * ex + cx) + (int64_t)gf.res[0] * ((2 * ey + cy) + (int64_t)gf.res[1] * (2 * ez + cz))];
    rc[e] = s;
}

template <int DIM>
__global__ void k_cell_prolong_add32(uwg_lgeom gf, uwg_lgeom gc, const float* xc, float* xf) {
    int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (e >= gf.n_el) return;
    int ex = (int)(e % gf.res[0]), ey = (int)((e / gf.res[0]) % gf.res[1]);
    int ez = DIM == 3 ? (int)(e / ((int64_t)gf.res[0] * gf.res[1])) : 0;
    xf[e] += xc[(ex >> 1) + (int64_t)gc.res[0] * ((ey >> 1) + (int64_t)gc.res[1] * (ez >> 1))];
}

#define DIMCALL(KERN, GRID, ...)                                                        \
    do {                                                                                 \
        if (c->dim == 3) KERN<3><<<GRID, 256, 0, c->stream>>>(__VA_ARGS__);             \
        else KERN<2><<<GRID, 256, 0, c->stream>>>(__VA_ARGS__);                         \
    } while (0)

int uwg_ops_G32(uwg_ctx* c, int l, const float* Dinv, const float* p, float* v) {
    uwg_lgeom g = uwg_level_geom(c, l);
    DIMCALL(k_gradG32, nblk(g.n_nodes), g, c->lev[l].bc, p, Dinv, v);
    UWG_CUDA(c, cudaGetLastError());
    return UWG_OK;
}
int uwg_ops_Gt32(uwg_ctx* c, int l, const float* v, float* q) {
    uwg_lgeom g = uwg_level_geom(c, l);
    DIMCALL(k_Gt32, nblk(g.n_el), g, c->lev[l].bc, v, q);
    UWG_CUDA(c, cudaGetLastError());
    return UWG_OK;
}
int uwg_ops_applyL32(uwg_ctx* c, int l, const float* Dinv, const float* p, float* q, float* vtmp) {
    int rc = uwg_ops_G32(c, l, Dinv, p, vtmp);
    return rc ? rc : uwg_ops_Gt32(c, l, vtmp, q);
}
int uwg_ops_Ldiag32(uwg_ctx* c, int l, const float* Dinv, float* out) {
    uwg_lgeom g = uwg_level_geom(c, l);
    DIMCALL(k_Ldiag32, nblk(g.n_el), g, c->lev[l].bc, Dinv, out);
    UWG_CUDA(c, cudaGetLastError());
    return UWG_OK;
}
int uwg_ops_winv(uwg_ctx* c, int l, float* out) {
    const uwg_level& L = c->lev[l];
    k_winv<<<nblk(L.n_dof), 256, 0, c->stream>>>(L.n_dof, L.diag64, L.bc, out);
    UWG_CUDA(c, cudaGetLastError());
    return UWG_OK;
}
int uwg_ops_cell_restrict32(uwg_ctx* c, int lc, const float* rf, float* rc_) {
    uwg_lgeom gf = uwg_level_geom(c, lc - 1), gc = uwg_level_geom(c, lc);
    DIMCALL(k_cell_restrict32, nblk(gc.n_el), gf, gc, rf, rc_);
    UWG_CUDA(c, cudaGetLastError());
    return UWG_OK;
}
int uwg_ops_cell_prolong_add32(uwg_ctx* c, int lc, const float* xc, float* xf) {
    uwg_lgeom gf = uwg_level_geom(c, lc - 1), gc = uwg_level_geom(c, lc);
    DIMCALL(k_cell_prolong_add32, nblk(gf.n_el), gf, gc, xc, xf);
    UWG_CUDA(c, cudaGetLastError());
    return UWG_OK;
}

// Pressure Laplacian of the scaled BFBt Schur preconditioner on level l:
// L p = G^T diag(K)^-1 G p (Dirichlet dofs excluded).
template <int DIM>
__global__ void k_applyGt_scaled(uwg_lgeom g, const uint8_t* bc, const double* diag, const double* u, double* q) {
    constexpr int NEN = DIM == 3 ? 8 : 4;
    int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (e >= g.n_el) return;
    int64_t nodes[8];
    double h[3];
    q1_elem(g, e, nodes, h);
    double s = 0.0;
    for (int n = 0; n < NEN; n++)
        for (int i = 0; i < DIM; i++) {
            int64_t dof = nodes[n] * DIM + i;
            if (bc[dof]) continue;
            double ge = 1.0;
            for (int d = 0; d < DIM; d++)
                if (d != i) ge *= 0.5 * h[d];
            ge *= ((n >> i) & 1) ? -1.0 : 1.0;
            s += ge * (u[dof] / diag[dof]);
        }
    q[e] = s;
}

template <int DIM>
__global__ void k_Ldiag(uwg_lgeom g, const uint8_t* bc, const double* diag, double* out) {
    constexpr int NEN = DIM == 3 ? 8 : 4;
    int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (e >= g.n_el) return;
    int64_t nodes[8];
    double h[3];
    q1_elem(g, e, nodes, h);
    double s = 0.0;
    for (int n = 0; n < NEN; n++)
        for (int i = 0; i < DIM; i++) {
            int64_t dof = nodes[n] * DIM + i;
            if (bc[dof]) continue;
            double ge = 1.0;
            for (int d = 0; d < DIM; d++)
                if (d != i) ge *= 0.5 * h[d];
            s += ge * ge / diag[dof];
        }
    out[e] = s > 0.0 ? s : 1.0;
}

template <int DIM>
__global__ void k_cell_restrict(uwg_lgeom gf, uwg_lgeom gc, const double* rf, double* rc) {
    int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (e >= gc.n_el) return;
    int ex = (int)(e % gc.res[0]), ey = (int)((e / gc.res[0]) % gc.res[1]);
    int ez = DIM == 3 ? (int)(e / ((int64_t)gc.res[0] * gc.res[1])) : 0;
    double s = 0.0;
    for (int cz = 0; cz < (DIM == 3 ? 2 : 1); cz++)
        for (int cy = 0; cy < 2; cy++)
            for (int cx = 0; cx < 2; cx++)
                s += rf[(2 * ex + cx) + (int64_t)gf.res[0] * ((2 * ey + cy) + (int64_t)gf.res[1] * (2 * ez + cz))];
    rc[e] = s;
}

template <int DIM>
__global__ void k_cell_prolong_add(uwg_lgeom gf, uwg_lgeom gc, const double* xc, double* xf) {
    int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (e >= gf.n_el) return;
    int ex = (int)(e % gf.res[0]), ey = (int)((e / gf.res[0]) % gf.res[1]);
    int ez = DIM == 3 ? (int)(e / ((int64_t)gf.res[0] * gf.res[1])) : 0;
    xf[e] += xc[(ex >> 1) + (int64_t)gc.res[0] * ((ey >> 1) + (int64_t)gc.res[1] * (ez >> 1))];
}

int uwg_ops_applyL(uwg_ctx* c, int l, const double* p, double* q, double* vtmp) {
    const uwg_level& L = c->lev[l];
    uwg_lgeom g = uwg_level_geom(c, l);
    if (c->dim == 3) {
        k_gradG_nodes<3><<<nblk(L.n_nodes), 256, 0, c->stream>>>(g, L.bc, p, L.diag64, vtmp);
        k_applyGt<3><<<nblk(L.n_el), 256, 0, c->stream>>>(g, L.bc, 0, vtmp, q);
    } else {
        k_gradG_nodes<2><<<nblk(L.n_nodes), 256, 0, c->stream>>>(g, L.bc, p, L.diag64, vtmp);
        k_applyGt<2><<<nblk(L.n_el), 256, 0, c->stream>>>(g, L.bc, 0, vtmp, q);
    }
    UWG_CUDA(c, cudaGetLastError());
    return UWG_OK;
}

int uwg_ops_Ldiag(uwg_ctx* c, int l, double* out) {
    const uwg_level& L = c->lev[l];
    uwg_lgeom g = uwg_level_geom(c, l);
    if (c->dim == 3) k_Ldiag<3><<<nblk(L.n_el), 256, 0, c->stream>>>(g, L.bc, L.diag64, out);
    else k_Ldiag<2><<<nblk(L.n_el), 256, 0, c->stream>>>(g, L.bc, L.diag64, out);
    UWG_CUDA(c, cudaGetLastError());
    return UWG_OK;
}

int uwg_ops_cell_restrict(uwg_ctx* c, int lc, const double* rf, double* rc) {
    uwg_lgeom gf = uwg_level_geom(c, lc - 1), gc = uwg_level_geom(c, lc);
    if (c->dim == 3) k_cell_restrict<3><<<nblk(gc.n_el), 256, 0, c->stream>>>(gf, gc, rf, rc);
    else k_cell_restrict<2><<<nblk(gc.n_el), 256, 0, c->stream>>>(gf, gc, rf, rc);
    UWG_CUDA(c, cudaGetLastError());
    return UWG_OK;
}

int uwg_ops_cell_prolong_add(uwg_ctx* c, int lc, const double* xc, double* xf) {
    uwg_lgeom gf = uwg_level_geom(c, lc - 1), gc = uwg_level_geom(c, lc);
    if (c->dim == 3) k_cell_prolong_add<3><<<nblk(gf.n_el), 256, 0, c->stream>>>(gf, gc, xc, xf);
    else k_cell_prolong_add<2><<<nblk(gf.n_el), 256, 0, c->stream>>>(gf, gc, xc, xf);
    UWG_CUDA(c, cudaGetLastError());
    return UWG_OK;
}

int uwg_ops_applyG(uwg_ctx* c, const double* p, double* y) {
    if (c->porder == 1) return uwg_q2_applyG(c, p, y);
    uwg_lgeom g = uwg_level_geom(c, 0);
    if (c->dim == 3) k_gradG_nodes<3><<<nblk(c->n_nodes), 256, 0, c->stream>>>(g, c->bc, p, nullptr, y);
    else k_gradG_nodes<2><<<nblk(c->n_nodes), 256, 0, c->stream>>>(g, c->bc, p, nullptr, y);
    UWG_CUDA(c, cudaGetLastError());
    return UWG_OK;
}

int uwg_ops_applyGt(uwg_ctx* c, const double* u, double* q) { return uwg_ops_applyGt_mode(c, u, q, 0); }

int uwg_ops_applyGt_mode(uwg_ctx* c, const double* u, double* q, int only_bc) {
    if (c->porder == 1) return uwg_q2_applyGt(c, u, q, only_bc);
    uwg_lgeom g = uwg_level_geom(c, 0);
    if (c->dim == 3) k_applyGt<3><<<nblk(c->n_el), 256, 0, c->stream>>>(g, c->bc, only_bc, u, q);
    else k_applyGt<2><<<nblk(c->n_el), 256, 0, c->stream>>>(g, c->bc, only_bc, u, q);
    UWG_CUDA(c, cudaGetLastError());
    return UWG_OK;
}

__global__ void k_schur_pc(int64_t n, const double* shat, const double* r, double* z) {
    int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i < n) z[i] = r[i] / shat[i];
}

int uwg_ops_schur_pc(uwg_ctx* c, const double* r, double* z) {
    if (c->porder == 1) return uwg_q2_schur_pc(c, r, z);
    k_schur_pc<<<nblk(c->n_pdof), 256, 0, c->stream>>>(c->n_pdof, c->Shat, r, z);
    UWG_CUDA(c, cudaGetLastError());
    return UWG_OK;
}

__global__ void k_pmul(int64_t n, const double* a, const double* x, double* y) {
    int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i < n) y[i] = a[i] * x[i];
}

int uwg_ops_apply_C(uwg_ctx* c, const double* p, double* q) {
    if (!c->Mp) { vk_zero<double>(c->stream, c->n_pdof, q); return UWG_OK; }
    k_pmul<<<nblk(c->n_pdof), 256, 0, c->stream>>>(c->n_pdof, c->Mp, p, q);
    UWG_CUDA(c, cudaGetLastError());
    return UWG_OK;
}

// ---------------------------------------------------------------------------
// Multigrid transfer (Q1 nested meshes).
// ---------------------------------------------------------------------------
template <typename T, int DIM>
__global__ void k_prolong_add(uwg_lgeom gf, uwg_lgeom gc, const uint8_t* bcf, const T* xc, T* xf) {
    int64_t nd = gf.n_nodes;
    int64_t n = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (n >= nd) return;
    int fi[3] = {(int)(n % gf.nx[0]), (int)((n / gf.nx[0]) % gf.nx[1]), DIM == 3 ? (int)(n / ((int64_t)gf.nx[0] * gf.nx[1])) : 0};
    int lo[3], hi[3];
    T wl[3], wh[3];
    for (int d = 0; d < 3; d++) {
        if (d >= DIM) { lo[d] = hi[d] = 0; wl[d] = 1; wh[d] = 0; continue; }
        if (fi[d] & 1) { lo[d] = fi[d] >> 1; hi[d] = lo[d] + 1; wl[d] = 0.5; wh[d] = 0.5; }
        else { lo[d] = hi[d] = fi[d] >> 1; wl[d] = 1; wh[d] = 0; }
    }
    T acc[3] = {0, 0, 0};
    for (int kz = 0; kz < (DIM == 3 ? 2 : 1); kz++)
        for (int ky = 0; ky < 2; ky++)
            for (int kx = 0; kx < 2; kx++) {
                T w = (kx ? wh[0] : wl[0]) * (ky ? wh[1] : wl[1]) * (DIM == 3 ? (kz ? wh[2] : wl[2]) : (T)1);
                if (w == (T)0) continue;
                int64_t cn = (kx ? hi[0] : lo[0]) + (int64_t)gc.nx[0] * ((ky ? hi[1] : lo[1]) + (int64_t)gc.nx[1] * (kz ? hi[2] : lo[2]));
                for (int c = 0; c < DIM; c++) acc[c] += w * xc[cn * DIM + c];
            }
    for (int c = 0; c < DIM; c++)
        if (!bcf[n * DIM + c]) xf[n * DIM + c] += acc[c];
}

template <typename T, int DIM>
__global__ void k_restrict(uwg_lgeom gf, uwg_lgeom gc, const uint8_t* bcf, const uint8_t* bcc, const T* rf, T* rc) {
    int64_t n = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (n >= gc.n_nodes) return;
    int ci[3] = {(int)(n % gc.nx[0]), (int)((n / gc.nx[0]) % gc.nx[1]), DIM == 3 ? (int)(n / ((int64_t)gc.nx[0] * gc.nx[1])) : 0};
    T acc[3] = {0, 0, 0};
    for (int dz = (DIM == 3 ? -1 : 0); dz <= (DIM == 3 ? 1 : 0); dz++)
        for (int dy = -1; dy <= 1; dy++)
            for (int dx = -1; dx <= 1; dx++) {
                int f[3] = {2 * ci[0] + dx, 2 * ci[1] + dy, 2 * ci[2] + dz};
                bool ok = true;
                for (int d = 0; d < DIM; d++) ok = ok && f[d] >= 0 && f[d] < gf.nx[d];
                if (!ok) continue;
                T w = (dx ? (T)0.5 : (T)1) * (dy ? (T)0.5 : (T)1) * (dz ? (T)0.5 : (T)1);
                int64_t fn = f[0] + (int64_t)gf.nx[0] * (f[1] + (int64_t)gf.nx[1] * f[2]);
                for (int c = 0; c < DIM; c++)
                    if (!bcf[fn * DIM + c]) acc[c] += w * rf[fn * DIM + c];
            }
    for (int c = 0; c < DIM; c++) rc[n * DIM + c] = bcc[n * DIM + c] ? (T)0 : acc[c];
}

template <typename T>
int uwg_ops_prolong_add(uwg_ctx* c, int lc, const T* xc, T* xf) {
    uwg_lgeom gf = uwg_level_geom(c, lc - 1), gc = uwg_level_geom(c, lc);
    if (c->dim == 3) k_prolong_add<T, 3><<<nblk(gf.n_nodes), 256, 0, c->stream>>>(gf, gc, c->lev[lc - 1].bc, xc, xf);
    else k_prolong_add<T, 2><<<nblk(gf.n_nodes), 256, 0, c->stream>>>(gf, gc, c->lev[lc - 1].bc, xc, xf);
    UWG_CUDA(c, cudaGetLastError());
    return UWG_OK;
}
template <typename T>
int uwg_ops_restrict(uwg_ctx* c, int lc, const T* rf, T* rc) {
    uwg_lgeom gf = uwg_level_geom(c, lc - 1), gc = uwg_level_geom(c, lc);
    if (c->dim == 3) k_restrict<T, 3><<<nblk(gc.n_nodes), 256, 0, c->stream>>>(gf, gc, c->lev[lc - 1].bc, c->lev[lc].bc, rf, rc);
    else k_restrict<T, 2><<<nblk(gc.n_nodes), 256, 0, c->stream>>>(gf, gc, c->lev[lc - 1].bc, c->lev[lc].bc, rf, rc);
    UWG_CUDA(c, cudaGetLastError());
    return UWG_OK;
}
template int uwg_ops_prolong_add<double>(uwg_ctx*, int, const double*, double*);
template int uwg_ops_prolong_add<float>(uwg_ctx*, int, const float*, float*);
template int uwg_ops_restrict<double>(uwg_ctx*, int, const double*, double*);
template int uwg_ops_restrict<float>(uwg_ctx*, int, const float*, float*);

// Coarsening of W: parent weights from the children's, separable 3x3 maps.
// Child points s in {-1,0,1} sit at parent coordinate (s + 2*delta - 1)/2.
__constant__ double c_T[2][3][3];   // [delta][child point][parent point]

template <int DIM>
__global__ void k_coarsen_W(uwg_lgeom gf, uwg_lgeom gc, const double* Wf, double* Wc) {
    constexpr int NQ = DIM == 3 ? 27 : 9;
    int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (e >= gc.n_el) return;
    int ex = (int)(e % gc.res[0]), ey = (int)((e / gc.res[0]) % gc.res[1]);
    int ez = DIM == 3 ? (int)(e / ((int64_t)gc.res[0] * gc.res[1])) : 0;
    double acc[NQ];
    for (int j = 0; j < NQ; j++) acc[j] = 0.0;
    for (int cz = 0; cz < (DIM == 3 ? 2 : 1); cz++)
        for (int cy = 0; cy < 2; cy++)
            for (int cx = 0; cx < 2; cx++) {
                int64_t fe = (2 * ex + cx) + (int64_t)gf.res[0] * ((2 * ey + cy) + (int64_t)gf.res[1] * (2 * ez + cz));
                double w[NQ], t1[NQ], t2[NQ];
                for (int j = 0; j < NQ; j++) w[j] = Wf[(int64_t)j * gf.n_el + fe];
                // x
                for (int k = 0; k < NQ / 3; k++)
                    for (int a = 0; a < 3; a++) {
                        double s = 0.0;
                        for (int b = 0; b < 3; b++) s += c_T[cx][b][a] * w[b + 3 * k];
                        t1[a + 3 * k] = s;
                    }
                // y
                for (int kz = 0; kz < (DIM == 3 ? 3 : 1); kz++)
                    for (int a = 0; a < 3; a++)
                        for (int ix = 0; ix < 3; ix++) {
                            double s = 0.0;
                            for (int b = 0; b < 3; b++) s += c_T[cy][b][a] * t1[ix + 3 * b + 9 * kz];
                            t2[ix + 3 * a + 9 * kz] = s;
                        }
                if (DIM == 3) {
                    for (int a = 0; a < 3; a++)
                        for (int ixy = 0; ixy < 9; ixy++) {
                            double s = 0.0;
                            for (int b = 0; b < 3; b++) s += c_T[cz][b][a] * t2[ixy + 9 * b];
                            acc[ixy + 9 * a] += s;
                        }
                } else {
                    for (int j = 0; j < NQ; j++) acc[j] += t2[j];
                }
            }
    for (int j = 0; j < NQ; j++) Wc[(int64_t)j * gc.n_el + e] = acc[j];
}

int uwg_ops_coarsen(uwg_ctx* c, int l) {
    static bool init = false;
    if (!init) {
        double T[2][3][3];
        for (int dl = 0; dl < 2; dl++)
            for (int b = 0; b < 3; b++) {
                double s = ((b - 1) + (2 * dl - 1)) * 0.5;
                T[dl][b][0] = 0.5 * s * (s - 1.0);
                T[dl][b][1] = 1.0 - s * s;
                T[dl][b][2] = 0.5 * s * (s + 1.0);
            }
        UWG_CUDA(c, cudaMemcpyToSymbol(c_T, T, sizeof(T)));
        init = true;
    }
    uwg_lgeom gf = uwg_level_geom(c, l), gc = uwg_level_geom(c, l + 1);
    if (c->dim == 3) k_coarsen_W<3><<<nblk(gc.n_el, 128), 128, 0, c->stream>>>(gf, gc, c->lev[l].W64, c->lev[l + 1].W64);
    else k_coarsen_W<2><<<nblk(gc.n_el, 128), 128, 0, c->stream>>>(gf, gc, c->lev[l].W64, c->lev[l + 1].W64);
    UWG_CUDA(c, cudaGetLastError());
    return UWG_OK;
}

__global__ void k_bc_coarsen(uwg_lgeom gf, uwg_lgeom gc, int dim, const uint8_t* bcf, uint8_t* bcc) {
    int64_t n = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (n >= gc.n_nodes) return;
    int ci[3] = {(int)(n % gc.nx[0]), (int)((n / gc.nx[0]) % gc.nx[1]), dim == 3 ? (int)(n / ((int64_t)gc.nx[0] * gc.nx[1])) : 0};
    int64_t fn = 2 * ci[0] + (int64_t)gf.nx[0] * (2 * ci[1] + (int64_t)gf.nx[1] * 2 * ci[2]);
    for (int c = 0; c < dim; c++) bcc[n * dim + c] = bcf[fn * dim + c];
}

int uwg_ops_bc_coarsen(uwg_ctx* c, int l) {
    uwg_lgeom gf = uwg_level_geom(c, l), gc = uwg_level_geom(c, l + 1);
    k_bc_coarsen<<<nblk(gc.n_nodes), 256, 0, c->stream>>>(gf, gc, c->dim, c->lev[l].bc, c->lev[l + 1].bc);
    UWG_CUDA(c, cudaGetLastError());
    return UWG_OK;
}

__global__ void k_to_f32(int64_t n, const double* a, float* b) {
    int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i < n) b[i] = (float)a[i];
}

int uwg_ops_level_setup(uwg_ctx* c, int l) {
    uwg_level& L = c->lev[l];
    uwg_lgeom g = uwg_level_geom(c, l);
    vk_zero<double>(c->stream, L.n_dof, L.diag64);
    if (L.order == 2) {
        int rc = uwg_q2_diag(c, l == 0 ? c->Shat : nullptr);
        if (rc) return rc;
        k_diag_bc<<<nblk(L.n_dof), 256, 0, c->stream>>>(L.n_dof, L.bc, L.diag64, L.diag32, nullptr);
        k_to_f32<<<nblk(L.n_el * L.nq), 256, 0, c->stream>>>(L.n_el * L.nq, L.W64, L.W32);
        UWG_CUDA(c, cudaGetLastError());
        return UWG_OK;
    }
    if (c->dim == 3) {
        // per-tile Dirichlet flags of the tiled apply (the mask of this level is final here)
        int64_t nt = uwg_ops_ktiles(L.res);
        if (!L.tile_bc) UWG_CUDA(c, cudaMalloc((void**)&L.tile_bc, nt));
        k_tile_bc_flags<<<(unsigned)nt, 256, 0, c->stream>>>(g, L.bc, L.tile_bc);
        UWG_CUDA(c, cudaGetLastError());
        if (l == 0) {
            // double-float copy of W for the refinement residual (without room for it the
            // residual uses the FP64 apply)
            const int64_t nw = (int64_t)27 * L.n_el;
            if (!L.Wdf && cudaMalloc((void**)&L.Wdf, sizeof(float2) * nw) != cudaSuccess) {
                cudaGetLastError();
                L.Wdf = nullptr;
            }
            if (L.Wdf) k_split_w_df<<<nblk(nw), 256, 0, c->stream>>>(nw, L.W64, L.Wdf);
            UWG_CUDA(c, cudaGetLastError());
        }
    }
    if (c->dim == 3) k_diag_q1<3><<<nblk(L.n_el), 256, 0, c->stream>>>(g, L.W64, L.bc, L.diag64, l == 0 ? c->Shat : nullptr, c->Mp);
    else k_diag_q1<2><<<nblk(L.n_el), 256, 0, c->stream>>>(g, L.W64, L.bc, L.diag64, l == 0 ? c->Shat : nullptr, c->Mp);
    UWG_CUDA(c, cudaGetLastError());
    k_diag_bc<<<nblk(L.n_dof), 256, 0, c->stream>>>(L.n_dof, L.bc, L.diag64, L.diag32, nullptr);
    int nq = c->dim == 3 ? 27 : 9;
    k_to_f32<<<nblk(L.n_el * nq), 256, 0, c->stream>>>(L.n_el * nq, L.W64, L.W32);
    UWG_CUDA(c, cudaGetLastError());
    return UWG_OK;
}

// ---------------------------------------------------------------------------
// Element matrices from W (diagnostics and the dense coarse operator).
// ---------------------------------------------------------------------------
template <int DIM>
__device__ void q1_Ke_from_W(const double* Wl, const double* h, double* Ke) {
    constexpr int NQ = DIM == 3 ? 27 : 9;
    constexpr int NEN = DIM == 3 ? 8 : 4;
    constexpr int ND = NEN * DIM;
    double hi[3] = {2.0 / h[0], 2.0 / h[1], DIM == 3 ? 2.0 / h[2] : 1.0};
    for (int i = 0; i < ND * ND; i++) Ke[i] = 0.0;
    for (int j = 0; j < NQ; j++) {
        int pt[3] = {j % 3, (j / 3) % 3, DIM == 3 ? j / 9 : 1};
        double gx[NEN][3];
        for (int n = 0; n < NEN; n++)
            for (int d = 0; d < DIM; d++) gx[n][d] = hi[d] * q1_lderiv<DIM>(n, d, pt);
        for (int a = 0; a < NEN; a++)
            for (int b = 0; b < NEN; b++) {
                double s2 = 0.0;
                for (int d = 0; d < DIM; d++) s2 += gx[a][d] * gx[b][d];
                for (int ci = 0; ci < DIM; ci++)
                    for (int cj = 0; cj < DIM; cj++) {
                        double v = gx[a][cj] * gx[b][ci] + (ci == cj ? s2 : 0.0);
                        Ke[(a * DIM + ci) * ND + b * DIM + cj] += Wl[j] * v;
                    }
            }
    }
}

template <int DIM>
__global__ void k_element_matrices(uwg_lgeom g, int64_t e, const double* W, const double* shat, double* Ke,
                                   double* Ge, double* Se) {
    constexpr int NQ = DIM == 3 ? 27 : 9;
    constexpr int NEN = DIM == 3 ? 8 : 4;
    int64_t nodes[8];
    double h[3], Wl[NQ];
    q1_elem(g, e, nodes, h);
    for (int j = 0; j < NQ; j++) Wl[j] = W[(int64_t)j * g.n_el + e];
    q1_Ke_from_W<DIM>(Wl, h, Ke);
    for (int n = 0; n < NEN; n++)
        for (int i = 0; i < DIM; i++) {
            double ge = 1.0;
            for (int d = 0; d < DIM; d++)
                if (d != i) ge *= 0.5 * h[d];
            Ge[n * DIM + i] = ge * (((n >> i) & 1) ? -1.0 : 1.0);
        }
    Se[0] = shat[e];
}

int uwg_ops_element_matrices(uwg_ctx* c, int64_t el, double* Ke, double* fe, double* Ge, double* Se) {
    int nd = c->dim * c->nen;
    if (c->order == 2) {
        if (fe) for (int i = 0; i < nd; i++) fe[i] = 0.0;   // element force is scattered at assembly
        return uwg_q2_element_matrices(c, el, Ke, Ge, Se);
    }
    double* buf = nullptr;
    UWG_CUDA(c, cudaMallocAsync((void**)&buf, sizeof(double) * (nd * nd + nd + 1), c->stream));
    uwg_lgeom g = uwg_level_geom(c, 0);
    if (c->dim == 3) k_element_matrices<3><<<1, 1, 0, c->stream>>>(g, el, c->lev[0].W64, c->Shat, buf, buf + nd * nd, buf + nd * nd + nd);
    else k_element_matrices<2><<<1, 1, 0, c->stream>>>(g, el, c->lev[0].W64, c->Shat, buf, buf + nd * nd, buf + nd * nd + nd);
    std::vector<double> h(nd * nd + nd + 1);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaMemcpyAsync(h.data(), buf, sizeof(double) * h.size(), cudaMemcpyDeviceToHost, c->stream);
    cudaFreeAsync(buf, c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) return uwg_set_error(c, UWG_ERR_CUDA, cudaGetErrorString(e));
    if (Ke) std::copy(h.begin(), h.begin() + nd * nd, Ke);
    if (Ge) std::copy(h.begin() + nd * nd, h.begin() + nd * nd + nd, Ge);
    if (Se) Se[0] = h[nd * nd + nd];
    if (fe) {
        for (int i = 0; i < nd; i++) fe[i] = 0.0;   // element force is scattered at assembly
    }
    return UWG_OK;
}

// Dense coarse operator: assemble from W, then Gauss-Jordan inverse in one block.
template <int DIM>
__global__ void k_dense_assemble(uwg_lgeom g, const double* W, const uint8_t* bc, int64_t n, double* A) {
    constexpr int NQ = DIM == 3 ? 27 : 9;
    constexpr int NEN = DIM == 3 ? 8 : 4;
    constexpr int ND = NEN * DIM;
    int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (e >= g.n_el) return;
    int64_t nodes[8];
    double h[3], Wl[NQ], Ke[ND * ND];
    q1_elem(g, e, nodes, h);
    for (int j = 0; j < NQ; j++) Wl[j] = W[(int64_t)j * g.n_el + e];
    q1_Ke_from_W<DIM>(Wl, h, Ke);
    for (int a = 0; a < ND; a++)
        for (int b = 0; b < ND; b++) {
            int64_t r = nodes[a / DIM] * DIM + a % DIM, cc = nodes[b / DIM] * DIM + b % DIM;
            if (bc[r] || bc[cc]) continue;
            atomicAdd(&A[r * n + cc], Ke[a * ND + b]);
        }
}

__global__ void k_dense_bcdiag(int64_t n, const uint8_t* bc, double* A) {
    int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i < n && bc[i]) A[i * n + i] = 1.0;
}

// In-place Gauss-Jordan inverse of an SPD matrix (no pivoting needed), one block.
__global__ void k_dense_invert(int64_t n, double* A, double* B) {
    // B <- I; eliminate column by column on [A | B]
    for (int64_t i = threadIdx.x; i < n * n; i += blockDim.x) B[i] = (i / n == i % n) ? 1.0 : 0.0;
    __syncthreads();
    for (int64_t k = 0; k < n; k++) {
        double piv = A[k * n + k];
        __syncthreads();
        for (int64_t j = threadIdx.x; j < n; j += blockDim.x) {
            A[k * n + j] /= piv;
            B[k * n + j] /= piv;
        }
        __syncthreads();
        for (int64_t idx = threadIdx.x; idx < n * n; idx += blockDim.x) {
            int64_t i = idx / n, j = idx % n;
            if (i == k) continue;
            double f = A[i * n + k];
            if (j != k) A[i * n + j] -= f * A[k * n + j];
            B[i * n + j] -= f * B[k * n + j];
        }
        __syncthreads();
        for (int64_t i = threadIdx.x; i < n; i += blockDim.x)
            if (i != k) A[i * n + k] = 0.0;
        __syncthreads();
    }
}

int uwg_ops_dense_matrix(uwg_ctx* c, int l, double* A) {
    uwg_level& L = c->lev[l];
    int64_t n = L.n_dof;
    uwg_lgeom g = uwg_level_geom(c, l);
    UWG_CUDA(c, cudaMemsetAsync(A, 0, sizeof(double) * n * n, c->stream));
    if (c->dim == 3) k_dense_assemble<3><<<nblk(L.n_el, 64), 64, 0, c->stream>>>(g, L.W64, L.bc, n, A);
    else k_dense_assemble<2><<<nblk(L.n_el, 64), 64, 0, c->stream>>>(g, L.W64, L.bc, n, A);
    k_dense_bcdiag<<<nblk(n), 256, 0, c->stream>>>(n, L.bc, A);
    UWG_CUDA(c, cudaGetLastError());
    return UWG_OK;
}

int uwg_ops_dense_coarse(uwg_ctx* c, int l) {
    uwg_level& L = c->lev[l];
    int64_t n = L.n_dof;
    if (n > 4096) return uwg_set_error(c, UWG_ERR_ARG, "coarsest multigrid level too large for a dense solve");
    uwg_lgeom g = uwg_level_geom(c, l);
    double* A = nullptr;
    UWG_CUDA(c, cudaMallocAsync((void**)&A, sizeof(double) * n * n, c->stream));
    UWG_CUDA(c, cudaMemsetAsync(A, 0, sizeof(double) * n * n, c->stream));
    if (c->dim == 3) k_dense_assemble<3><<<nblk(L.n_el, 64), 64, 0, c->stream>>>(g, L.W64, L.bc, n, A);
    else k_dense_assemble<2><<<nblk(L.n_el, 64), 64, 0, c->stream>>>(g, L.W64, L.bc, n, A);
    k_dense_bcdiag<<<nblk(n), 256, 0, c->stream>>>(n, L.bc, A);
    k_dense_invert<<<1, 1024, 0, c->stream>>>(n, A, L.cinv64);
    k_to_f32<<<nblk(n * n), 256, 0, c->stream>>>(n * n, L.cinv64, L.cinv32);
    cudaError_t e = cudaGetLastError();
    cudaFreeAsync(A, c->stream);
    if (e != cudaSuccess) return uwg_set_error(c, UWG_ERR_CUDA, cudaGetErrorString(e));
    return UWG_OK;
}

template <typename T>
__global__ void k_dense_mv(int64_t n, const T* Ainv, const T* b, T* x) {
    int64_t i = blockIdx.x * (int64_t)(blockDim.x / 32) + (threadIdx.x >> 5);
    int lane = threadIdx.x & 31;
    if (i >= n) return;
    T s = 0;
    for (int64_t j = lane; j < n; j += 32) s += Ainv[i * n + j] * b[j];
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if (lane == 0) x[i] = s;
}

// C = [A | I] (n x 2n, row-major) in both ping-pong buffers
__global__ void k_gj_init(int64_t n, const double* __restrict__ A, double* __restrict__ C0, double* __restrict__ C1) {
    const int64_t i = blockIdx.y, j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (j >= 2 * n) return;
    const double v = j < n ? A[i * n + j] : (j - n == i ? 1.0 : 0.0);
    C0[i * 2 * n + j] = v;
    C1[i * 2 * n + j] = v;
}

// Gauss-Jordan pivot k on C = [A | B]: only columns k .. n + k change (A's
// columns left of k are unit vectors, B's columns right of k are still the
// identity's), so the grid covers that window; row i per blockIdx.y, one
// reciprocal of the pivot per CTA.
__global__ void k_gj_win(int64_t n, int64_t k, const double* __restrict__ Ci, double* __restrict__ Co) {
    __shared__ double inv;
    if (threadIdx.x == 0) inv = 1.0 / Ci[k * 2 * n + k];
    __syncthreads();
    const int64_t i = blockIdx.y, j = k + blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (j > n + k) return;
    const int64_t ld = 2 * n;
    const double rk = Ci[k * ld + j] * inv;
    Co[i * ld + j] = (i == k) ? rk : Ci[i * ld + j] - Ci[i * ld + k] * rk;
}

__global__ void k_gj_extract(int64_t n, const double* __restrict__ C, double* __restrict__ B) {
    const int64_t i = blockIdx.y, j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (j < n) B[i * n + j] = C[i * 2 * n + n + j];
}

// B = A^-1 (the one-CTA path overwrites A).  Small matrices in one CTA; larger ones one
// grid-wide launch per pivot (a single CTA took 0.6 s at n = 1024).
int uwg_ops_dense_invert(uwg_ctx* c, int64_t n, double* A, double* B) {
    if (n <= 256) {
        k_dense_invert<<<1, 1024, 0, c->stream>>>(n, A, B);
        UWG_CUDA(c, cudaGetLastError());
        return UWG_OK;
    }
    return uwg_ops_dense_invert_grid(c, n, A, B);
}
int uwg_ops_dense_invert_grid(uwg_ctx* c, int64_t n, double* A, double* B) {
    if (n < 1 || n > 65535) return uwg_set_error(c, UWG_ERR_ARG, "dense inverse: n out of range");
    double *C0 = nullptr, *C1 = nullptr;
    UWG_CUDA(c, cudaMallocAsync((void**)&C0, sizeof(double) * 2 * n * n, c->stream));
    UWG_CUDA(c, cudaMallocAsync((void**)&C1, sizeof(double) * 2 * n * n, c->stream));
    k_gj_init<<<dim3(nblk(2 * n), (unsigned)n), 256, 0, c->stream>>>(n, A, C0, C1);
    double *ci = C0, *co = C1;
    const dim3 grid(nblk(n + 1), (unsigned)n);
    for (int64_t k = 0; k < n; k++) {
        k_gj_win<<<grid, 256, 0, c->stream>>>(n, k, ci, co);
        std::swap(ci, co);
    }
    k_gj_extract<<<dim3(nblk(n), (unsigned)n), 256, 0, c->stream>>>(n, ci, B);
    cudaFreeAsync(C0, c->stream);
    cudaFreeAsync(C1, c->stream);
    UWG_CUDA(c, cudaGetLastError());
    return UWG_OK;
}
int uwg_ops_to_f32(uwg_ctx* c, int64_t n, const double* a, float* b) {
    k_to_f32<<<nblk(n), 256, 0, c->stream>>>(n, a, b);
    UWG_CUDA(c, cudaGetLastError());
    return UWG_OK;
}
int uwg_ops_dense_mv32(uwg_ctx* c, int64_t n, const float* Ainv, const float* b, float* x) {
    k_dense_mv<float><<<nblk(n * 32, 256), 256, 0, c->stream>>>(n, Ainv, b, x);
    UWG_CUDA(c, cudaGetLastError());
    return UWG_OK;
}

template <typename T>
int uwg_ops_dense_solve(uwg_ctx* c, int l, const T* b, T* x) {
    uwg_level& L = c->lev[l];
    const T* Ainv;
    if constexpr (sizeof(T) == 8) Ainv = (const T*)L.cinv64; else Ainv = (const T*)L.cinv32;
    k_dense_mv<T><<<nblk(L.n_dof * 32, 256), 256, 0, c->stream>>>(L.n_dof, Ainv, b, x);
    UWG_CUDA(c, cudaGetLastError());
    return UWG_OK;
}
template int uwg_ops_dense_solve<double>(uwg_ctx*, int, const double*, double*);
template int uwg_ops_dense_solve<float>(uwg_ctx*, int, const float*, float*);

int uwg_ops_assemble(uwg_ctx* c, const int32_t* off, const int32_t* list, const double* ip_xi,
                     const double* ip_w, const double* eta_p, const double* body_p, const double* lambda_p) {
    if (c->order == 2) {
        if (lambda_p) return uwg_set_error(c, UWG_ERR_ARG, "compressibility is not available for Q2/dPc1");
        return uwg_q2_assemble(c, off, list, ip_xi, ip_w, eta_p, body_p);
    }
    uwg_lgeom g = uwg_level_geom(c, 0);
    vk_zero<double>(c->stream, c->n_vdof, c->f);
    if (c->dim == 3)
        k_assemble_q1<3><<<nblk(c->n_el, 128), 128, 0, c->stream>>>(g, off, list, ip_xi, ip_w, eta_p, body_p, lambda_p,
                                                                     c->lev[0].W64, c->f, c->Mp);
    else
        k_assemble_q1<2><<<nblk(c->n_el, 128), 128, 0, c->stream>>>(g, off, list, ip_xi, ip_w, eta_p, body_p, lambda_p,
                                                                     c->lev[0].W64, c->f, c->Mp);
    UWG_CUDA(c, cudaGetLastError());
    return UWG_OK;
}

// ---------------------------------------------------------------------------
// Vector kernels
// ---------------------------------------------------------------------------
template <typename T> __global__ void vk_copy_k(int64_t n, const T* x, T* y) {
    int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i < n) y[i] = x[i];
}
template <typename A, typename B> __global__ void vk_convert_k(int64_t n, const A* x, B* y) {
    int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i < n) y[i] = (B)x[i];
}
template <typename T> __global__ void vk_axpy_k(int64_t n, T a, const T* x, T* y) {
    int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i < n) y[i] += a * x[i];
}
template <typename T> __global__ void vk_axpby_k(int64_t n, T a, const T* x, T b, T* y) {
    int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i < n) y[i] = a * x[i] + b * y[i];
}
template <typename T> __global__ void vk_scale_k(int64_t n, T a, T* y) {
    int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i < n) y[i] *= a;
}
// One Chebyshev step: r = b - t (t may be null: r = b); d = a*(r/diag) + c*d; x (+)= d
template <typename T> __global__ void vk_cheb_k(int64_t n, const T* b, const T* t, const T* diag, T a, T c,
                                             T* d, T* x, int first, int x_zero) {
    int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    T r = t ? b[i] - t[i] : b[i];
    T dn = a * (r / diag[i]);
    if (!first) dn += c * d[i];
    d[i] = dn;
    x[i] = x_zero ? dn : x[i] + dn;
}
template <typename T> __global__ void vk_mask_k(int64_t n, const uint8_t* bc, T* y) {
    int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i < n && bc[i]) y[i] = 0;
}
template <typename T> __global__ void vk_pdiv_k(int64_t n, const T* x, const T* d, T* y) {
    int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i < n) y[i] = x[i] / d[i];
}

template <typename T> void vk_copy(cudaStream_t s, int64_t n, const T* x, T* y) { if (n) vk_copy_k<T><<<nblk(n), 256, 0, s>>>(n, x, y); }
template <typename A, typename B> void vk_convert(cudaStream_t s, int64_t n, const A* x, B* y) { if (n) vk_convert_k<A, B><<<nblk(n), 256, 0, s>>>(n, x, y); }
template <typename T> void vk_axpy(cudaStream_t s, int64_t n, T a, const T* x, T* y) { if (n) vk_axpy_k<T><<<nblk(n), 256, 0, s>>>(n, a, x, y); }
template <typename T> void vk_axpby(cudaStream_t s, int64_t n, T a, const T* x, T b, T* y) { if (n) vk_axpby_k<T><<<nblk(n), 256, 0, s>>>(n, a, x, b, y); }
template <typename T> void vk_scale(cudaStream_t s, int64_t n, T a, T* y) { if (n) vk_scale_k<T><<<nblk(n), 256, 0, s>>>(n, a, y); }
template <typename T> void vk_zero(cudaStream_t s, int64_t n, T* y) { if (n) cudaMemsetAsync(y, 0, sizeof(T) * n, s); }
template <typename T> void vk_mask(cudaStream_t s, int64_t n, const uint8_t* bc, T* y) { if (n) vk_mask_k<T><<<nblk(n), 256, 0, s>>>(n, bc, y); }
__global__ void vk_mulmask_k(int64_t n, const float* w, float* y) {
    int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i < n) y[i] *= w[i];
}
// y *= w (w is zero on Dirichlet dofs)
void vk_pointwise_mul_mask(cudaStream_t s, int64_t n, const float* w, float* y) {
    if (n) vk_mulmask_k<<<nblk(n), 256, 0, s>>>(n, w, y);
}
template <typename T> void vk_cheb(cudaStream_t s, int64_t n, const T* b, const T* t, const T* diag, T a, T c, T* d,
                                   T* x, int first, int x_zero) {
    if (n) vk_cheb_k<T><<<nblk(n), 256, 0, s>>>(n, b, t, diag, a, c, d, x, first, x_zero);
}
template void vk_cheb<double>(cudaStream_t, int64_t, const double*, const double*, const double*, double, double,
                              double*, double*, int, int);
template void vk_cheb<float>(cudaStream_t, int64_t, const float*, const float*, const float*, float, float, float*,
                             float*, int, int);
template <typename T> void vk_pointwise_div(cudaStream_t s, int64_t n, const T* x, const T* d, T* y) { if (n) vk_pdiv_k<T><<<nblk(n), 256, 0, s>>>(n, x, d, y); }

template void vk_copy<double>(cudaStream_t, int64_t, const double*, double*);
template void vk_copy<float>(cudaStream_t, int64_t, const float*, float*);
template void vk_convert<double, float>(cudaStream_t, int64_t, const double*, float*);
template void vk_convert<float, double>(cudaStream_t, int64_t, const float*, double*);
template void vk_axpy<double>(cudaStream_t, int64_t, double, const double*, double*);
template void vk_axpy<float>(cudaStream_t, int64_t, float, const float*, float*);
template void vk_axpby<double>(cudaStream_t, int64_t, double, const double*, double, double*);
template void vk_axpby<float>(cudaStream_t, int64_t, float, const float*, float, float*);
template void vk_scale<double>(cudaStream_t, int64_t, double, double*);
template void vk_scale<float>(cudaStream_t, int64_t, float, float*);
template void vk_zero<double>(cudaStream_t, int64_t, double*);
template void vk_zero<float>(cudaStream_t, int64_t, float*);
template void vk_mask<double>(cudaStream_t, int64_t, const uint8_t*, double*);
template void vk_mask<float>(cudaStream_t, int64_t, const uint8_t*, float*);
template void vk_pointwise_div<double>(cudaStream_t, int64_t, const double*, const double*, double*);
template void vk_pointwise_div<float>(cudaStream_t, int64_t, const float*, const float*, float*);

// Dot products: block partial sums in double, then atomics into dst.
struct dot_ptrs { const void* a[4]; const void* b[4]; };

template <typename T>
__global__ void vk_dots_k(int64_t n, int k, dot_ptrs P, double* dst) {
    __shared__ double sm[4][32];
    // per-thread partial sums in the vectors' own precision (a few dozen terms;
    // FP64 arithmetic is scarce on this GPU), FP64 from the warp reduction on
    T part[4] = {0, 0, 0, 0};
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        for (int j = 0; j < k; j++) part[j] += ((const T*)P.a[j])[i] * ((const T*)P.b[j])[i];
    double acc[4] = {(double)part[0], (double)part[1], (double)part[2], (double)part[3]};
    int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    for (int j = 0; j < k; j++) {
        double v = acc[j];
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
        if (lane == 0) sm[j][w] = v;
    }
    __syncthreads();
    if (w == 0) {
        for (int j = 0; j < k; j++) {
            double v = lane < (int)(blockDim.x >> 5) ? sm[j][lane] : 0.0;
            for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
            if (lane == 0) atomicAdd(&dst[j], v);
        }
    }
}

template <typename T>
void vk_dots(cudaStream_t s, int64_t n, int k, const T* const* a, const T* const* b, double* dst) {
    dot_ptrs P;
    for (int j = 0; j < 4; j++) { P.a[j] = j < k ? a[j] : nullptr; P.b[j] = j < k ? b[j] : nullptr; }
    cudaMemsetAsync(dst, 0, sizeof(double) * k, s);
    unsigned nb = std::min<unsigned>(nblk(n, 256), 152u * 8u);
    if (nb == 0) nb = 1;
    vk_dots_k<T><<<nb, 256, 0, s>>>(n, k, P, dst);
}
template void vk_dots<double>(cudaStream_t, int64_t, int, const double* const*, const double* const*, double*);
template void vk_dots<float>(cudaStream_t, int64_t, int, const float* const*, const float* const*, double*);

#define MDOT_MAX 64
struct mdot_ptrs { const double* v[MDOT_MAX]; };

__global__ void vk_mdot_k(int64_t n, int k, mdot_ptrs P, const double* w, double* dst) {
    // one block-column of vectors per blockIdx.y
    __shared__ double sm[32];
    int j = blockIdx.y;
    double acc = 0.0;
    const double* v = P.v[j];
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        acc += v[i] * w[i];
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    int lane = threadIdx.x & 31, wi = threadIdx.x >> 5;
    if (lane == 0) sm[wi] = acc;
    __syncthreads();
    if (wi == 0) {
        acc = lane < (int)(blockDim.x >> 5) ? sm[lane] : 0.0;
        for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
        if (lane == 0) atomicAdd(&dst[j], acc);
    }
}

void vk_mdot(cudaStream_t s, int64_t n, int k, const double* const* V, const double* w, double* dst) {
    mdot_ptrs P;
    for (int j = 0; j < MDOT_MAX; j++) P.v[j] = j < k ? V[j] : nullptr;
    cudaMemsetAsync(dst, 0, sizeof(double) * k, s);
    unsigned nb = std::min<unsigned>(nblk(n, 256), 256u);
    if (nb == 0) nb = 1;
    vk_mdot_k<<<dim3(nb, k), 256, 0, s>>>(n, k, P, w, dst);
}

__global__ void vk_maxpy_k(int64_t n, int k, mdot_ptrs P, const double* coef, double* y) {
    int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    double s = 0.0;
    for (int j = 0; j < k; j++) s += coef[j] * P.v[j][i];
    y[i] += s;
}

// y += sum_j coef[j] V_j  (coef on the device)
void vk_maxpy(cudaStream_t s, int64_t n, int k, const double* coef_dev, const double* const* V, double* y) {
    mdot_ptrs P;
    for (int j = 0; j < MDOT_MAX; j++) P.v[j] = j < k ? V[j] : nullptr;
    if (n && k) vk_maxpy_k<<<nblk(n), 256, 0, s>>>(n, k, P, coef_dev, y);
}
