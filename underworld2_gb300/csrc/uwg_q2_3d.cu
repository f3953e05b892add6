// 3D Q2/dPc1 operators: triquadratic velocity (27 nodes), linear discontinuous
// pressure (4 coefficients per element, TrilinearInnerElType.c:202-215).
//
// The 2D design carried to 3D:
// * Viscous operator.  Every entry of the PIC integrand B^T D(eta) B of a Q2
//   element is a polynomial of degree <= 4 per axis on an affine element, so
//   5-point tensor Lagrange interpolation on {-1,-1/2,0,1/2,1}^3 reproduces it:
//       W_j = sum_q eta_q w_q detJ L_j(xi_q)   (125 weights per element),
//   and K_e u_e is evaluated on that 5x5x5 grid, sum-factorised axis by axis.
//   Level 1 of the velocity multigrid is the Q1 mesh on the same elements; its
//   operator is the Galerkin product P^T K P exactly, i.e. the Q1 PIC integral
//   with the 3-point weights of the same particles.
// * Gradient: G_e[(A,i)][k] = -int dN_A/dx_i M_k (GradientStiffnessMatrixTerm.c
//   :189-218) = -(prod_{j != i} h_j/2) times a reference integral, tabulated once.
// * Schur preconditioner: the reference's Uzawa term S^_e = G_e^T diag(K_e)^-1 G_e
//   (UzawaPreconditionerTerm.c:124-207), a 4x4 block per element, stored inverted
//   (the ILU(0) of a block-diagonal matrix is its exact inverse).
//
// The apply keeps one element per thread: the element's velocities are staged
// in shared memory, and each output component I is produced in its own pass over
// the 125 points, so that the accumulators of one component, not three, stay in
// registers; a pass evaluates only the five gradient entries its stresses
// sigma_Ij = w (d_j u_I + d_I u_j) read.
#include <cmath>
#include <vector>

#include "uwg_ops.cuh"

namespace {

inline unsigned nblk(int64_t n, int t = 256) { return (unsigned)((n + t - 1) / t); }

// 1D quadratic basis (nodes -1, 0, 1) and its derivative at {-1,-1/2,0,1/2,1}
__constant__ double c3_B5[5][3] = {{1.0, 0.0, 0.0}, {0.375, 0.75, -0.125}, {0.0, 1.0, 0.0},
                                   {-0.125, 0.75, 0.375}, {0.0, 0.0, 1.0}};
__constant__ double c3_D5[5][3] = {{-1.5, 2.0, -0.5}, {-1.0, 1.0, 0.0}, {-0.5, 0.0, 0.5},
                                   {0.0, -1.0, 1.0}, {0.5, -2.0, 1.5}};
__constant__ float c3_B5f[5][3] = {{1.0f, 0.0f, 0.0f}, {0.375f, 0.75f, -0.125f}, {0.0f, 1.0f, 0.0f},
                                   {-0.125f, 0.75f, 0.375f}, {0.0f, 0.0f, 1.0f}};
__constant__ float c3_D5f[5][3] = {{-1.5f, 2.0f, -0.5f}, {-1.0f, 1.0f, 0.0f}, {-0.5f, 0.0f, 0.5f},
                                   {0.0f, -1.0f, 1.0f}, {0.5f, -2.0f, 1.5f}};
// reference gradient integrals: c3_GR[i][A][k] = int dN_A/dxi_i M_k over [-1,1]^3
__constant__ double c3_GR[3][27][4];

template <typename T> __device__ __forceinline__ T B5(int p, int a);
template <typename T> __device__ __forceinline__ T D5(int p, int a);
template <> __device__ __forceinline__ double B5<double>(int p, int a) { return c3_B5[p][a]; }
template <> __device__ __forceinline__ double D5<double>(int p, int a) { return c3_D5[p][a]; }
template <> __device__ __forceinline__ float B5<float>(int p, int a) { return c3_B5f[p][a]; }
template <> __device__ __forceinline__ float D5<float>(int p, int a) { return c3_D5f[p][a]; }

__device__ __forceinline__ void q2e3(const uwg_lgeom& g, int64_t e, int* ex, double* h) {
    ex[0] = (int)(e % g.res[0]);
    ex[1] = (int)((e / g.res[0]) % g.res[1]);
    ex[2] = (int)(e / ((int64_t)g.res[0] * g.res[1]));
    for (int d = 0; d < 3; d++) h[d] = g.ax[d][2 * ex[d] + 2] - g.ax[d][2 * ex[d]];
}
__device__ __forceinline__ int64_t q2node3(const uwg_lgeom& g, const int* ex, int A) {
    const int a = A % 3, b = (A / 3) % 3, c = A / 9;
    return (2 * ex[0] + a) + (int64_t)g.nx[0] * ((2 * ex[1] + b) + (int64_t)g.nx[1] * (2 * ex[2] + c));
}

__device__ __forceinline__ double lag5v(double s, int j) {
    const double n[5] = {-1.0, -0.5, 0.0, 0.5, 1.0};
    double v = 1.0;
#pragma unroll
    for (int k = 0; k < 5; k++)
        if (k != j) v *= (s - n[k]) / (n[j] - n[k]);
    return v;
}
__device__ __forceinline__ double lag3v(double s, int j) {
    return j == 0 ? 0.5 * s * (s - 1.0) : (j == 1 ? 1.0 - s * s : 0.5 * s * (s + 1.0));
}

// PIC assembly, one warp per element: lane l owns W125 entries l, l+32, l+64,
// l+96, the Q1 weight l (< 27) and body-force entries l, l+32, l+64 (< 81).
// The 15 5-point and 9 3-point Lagrange values of each particle are computed by
// one lane each and broadcast.
__global__ void k_assemble_q2_3d(uwg_lgeom g, const int32_t* off, const int32_t* list, const double* ip_xi,
                                 const double* ip_w, const double* eta_p, const double* body_p, double* W125,
                                 double* W27, double* f) {
    const int lane = threadIdx.x & 31;
    const int64_t e = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    if (e >= g.n_el) return;   // warp-uniform
    int ex[3];
    double h[3];
    q2e3(g, e, ex, h);
    const double detJ = (h[0] * 0.5) * (h[1] * 0.5) * (h[2] * 0.5);
    double w125[4] = {0.0, 0.0, 0.0, 0.0}, w27 = 0.0, fe[3] = {0.0, 0.0, 0.0};
    for (int32_t s = off[e]; s < off[e + 1]; s++) {
        const int32_t p = list[s];
        double v = 0.0;
        if (lane < 15) v = lag5v(ip_xi[(int64_t)s * 3 + lane / 5], lane % 5);
        else if (lane < 24) v = lag3v(ip_xi[(int64_t)s * 3 + (lane - 15) / 3], (lane - 15) % 3);
        const double wd = ip_w[s] * detJ, cf = eta_p[p] * wd;
#pragma unroll
        for (int m = 0; m < 4; m++) {
            const int j = lane + 32 * m;
            const int jj = j < 125 ? j : 0;
            const double lx = __shfl_sync(0xffffffffu, v, jj % 5);
            const double ly = __shfl_sync(0xffffffffu, v, 5 + (jj / 5) % 5);
            const double lz = __shfl_sync(0xffffffffu, v, 10 + jj / 25);
            if (j < 125) w125[m] += cf * lx * ly * lz;
        }
        {
            const int jj = lane < 27 ? lane : 0;
            const double lx = __shfl_sync(0xffffffffu, v, 15 + jj % 3);
            const double ly = __shfl_sync(0xffffffffu, v, 18 + (jj / 3) % 3);
            const double lz = __shfl_sync(0xffffffffu, v, 21 + jj / 9);
            if (lane < 27) w27 += cf * lx * ly * lz;
        }
        if (body_p) {
#pragma unroll
            for (int m = 0; m < 3; m++) {
                const int k = lane + 32 * m;
                const int A = (k < 81 ? k : 0) / 3;
                const double nx = __shfl_sync(0xffffffffu, v, 15 + A % 3);
                const double ny = __shfl_sync(0xffffffffu, v, 18 + (A / 3) % 3);
                const double nz = __shfl_sync(0xffffffffu, v, 21 + A / 9);
                if (k < 81) fe[m] += wd * body_p[(int64_t)p * 3 + k % 3] * (nx * ny * nz);
            }
        }
    }
#pragma unroll
    for (int m = 0; m < 4; m++)
        if (lane + 32 * m < 125) W125[(int64_t)(lane + 32 * m) * g.n_el + e] = w125[m];
    if (lane < 27) W27[(int64_t)lane * g.n_el + e] = w27;
    if (body_p)
#pragma unroll
        for (int m = 0; m < 3; m++) {
            const int k = lane + 32 * m;
            if (k < 81) atomicAdd(&f[q2node3(g, ex, k / 3) * 3 + k % 3], fe[m]);
        }
}

// One output component I of y += K x for the thread's element.  sigma_Ij =
// w (d_j u_I + d_I u_j) needs five gradient entries per point: d_j u_I (three)
// and d_I u_c for the two other components, so the forward passes carry the
// value/derivative planes of component I and only the I-direction planes of
// the others.  The x-direction point loop is unrolled; z and y run as loops.
template <typename T, int BS, int I>
__device__ __forceinline__ void q2_3d_apply_component(const uwg_lgeom& g, const T* us, const T* __restrict__ Wp,
                                                      int64_t st, const T* sc, const int* ex, uint32_t fb, T* y) {
    constexpr int C1 = (I + 1) % 3, C2 = (I + 2) % 3;
    const int tid = threadIdx.x;
    T out[27];
#pragma unroll
    for (int A = 0; A < 27; A++) out[A] = (T)0;
#pragma unroll 1
    for (int r = 0; r < 5; r++) {
        // z stage: value (tI) and z derivative (sI) of u_I; the I-direction plane of u_C1, u_C2
        T tI[9], sI[9], o1[9], o2[9];
#pragma unroll
        for (int ab = 0; ab < 9; ab++) {
            T t = 0, sd = 0, v1 = 0, v2 = 0;
#pragma unroll
            for (int k = 0; k < 3; k++) {
                const T* un = us + ((ab + 9 * k) * 3) * BS + tid;
                const T uI = un[I * BS], u1 = un[C1 * BS], u2 = un[C2 * BS];
                const T bz = B5<T>(r, k), dz = D5<T>(r, k);
                const T oz = I == 2 ? dz : bz;
                t += bz * uI;
                sd += dz * uI;
                v1 += oz * u1;
                v2 += oz * u2;
            }
            tI[ab] = t;
            sI[ab] = sd;
            o1[ab] = v1;
            o2[ab] = v2;
        }
        T P1[9], P3[9];
#pragma unroll
        for (int k = 0; k < 9; k++) P1[k] = P3[k] = (T)0;
#pragma unroll 1
        for (int q = 0; q < 5; q++) {
            // y stage
            T A1[3], A2[3], A3[3], O1[3], O2[3];
#pragma unroll
            for (int a = 0; a < 3; a++) {
                T v1 = 0, v2 = 0, v3 = 0, w1 = 0, w2 = 0;
#pragma unroll
                for (int b = 0; b < 3; b++) {
                    const T by = B5<T>(q, b), dy = D5<T>(q, b);
                    const T oy = I == 1 ? dy : by;
                    v1 += by * tI[a + 3 * b];
                    v2 += dy * tI[a + 3 * b];
                    v3 += by * sI[a + 3 * b];
                    w1 += oy * o1[a + 3 * b];
                    w2 += oy * o2[a + 3 * b];
                }
                A1[a] = v1;
                A2[a] = v2;
                A3[a] = v3;
                O1[a] = w1;
                O2[a] = w2;
            }
            T L1[3] = {0, 0, 0}, L2[3] = {0, 0, 0}, L3[3] = {0, 0, 0};
#pragma unroll
            for (int p = 0; p < 5; p++) {
                // x stage: the five gradient entries at point (p, q, r)
                T gI[3], h1 = 0, h2 = 0;
                {
                    T d0 = 0, d1 = 0, d2 = 0;
#pragma unroll
                    for (int a = 0; a < 3; a++) {
                        const T bx = B5<T>(p, a), dx = D5<T>(p, a);
                        const T ox = I == 0 ? dx : bx;
                        d0 += dx * A1[a];
                        d1 += bx * A2[a];
                        d2 += bx * A3[a];
                        h1 += ox * O1[a];
                        h2 += ox * O2[a];
                    }
                    gI[0] = sc[0] * d0;
                    gI[1] = sc[1] * d1;
                    gI[2] = sc[2] * d2;
                    h1 *= sc[I];
                    h2 *= sc[I];
                }
                const T w = Wp[(int64_t)(p + 5 * q + 25 * r) * st];
                T sg[3];
                sg[I] = w * (gI[I] + gI[I]);
                sg[C1] = w * (gI[C1] + h1);
                sg[C2] = w * (gI[C2] + h2);
#pragma unroll
                for (int a = 0; a < 3; a++) {
                    L1[a] += D5<T>(p, a) * sg[0];
                    L2[a] += B5<T>(p, a) * sg[1];
                    L3[a] += B5<T>(p, a) * sg[2];
                }
            }
#pragma unroll
            for (int b = 0; b < 3; b++)
#pragma unroll
                for (int a = 0; a < 3; a++) {
                    P1[a + 3 * b] += B5<T>(q, b) * (sc[0] * L1[a]) + D5<T>(q, b) * (sc[1] * L2[a]);
                    P3[a + 3 * b] += B5<T>(q, b) * (sc[2] * L3[a]);
                }
        }
#pragma unroll
        for (int c = 0; c < 3; c++)
#pragma unroll
            for (int ab = 0; ab < 9; ab++) out[ab + 9 * c] += B5<T>(r, c) * P1[ab] + D5<T>(r, c) * P3[ab];
    }
#pragma unroll
    for (int A = 0; A < 27; A++)
        if (!((fb >> A) & 1u)) atomicAdd(&y[q2node3(g, ex, A) * 3 + I], out[A]);
}

// Asynchronous copy of one FP32 or FP64 value into shared memory.
template <int BYTES>
__device__ __forceinline__ void q2_cp_async(void* smem, const void* gmem) {
    const unsigned sa = (unsigned)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.ca.shared.global [%0], [%1], %2;\n" ::"r"(sa), "l"(gmem), "n"(BYTES));
}

// Dynamic shared memory of the apply: the element's 81 nodal values and its
// 125 weights for each of the BS threads (thread-fastest, conflict-free).
template <typename T, int BS>
constexpr size_t q2_3d_apply_smem() { return (size_t)(81 + 125) * BS * sizeof(T); }

// y += K x over free dofs, one element per thread (see the file header).  The
// 125 weights of the thread's element are copied to shared memory with
// cp.async while the nodal values are gathered, so the point loops read them
// without waiting on DRAM; every thread reads only what it copied itself.
template <typename T, int BS>
__global__ void __launch_bounds__(BS) k_applyK_q2_3d(uwg_lgeom g, const T* __restrict__ W,
                                                     const uint8_t* __restrict__ bc, bool mask_in,
                                                     const T* __restrict__ x, T* y) {
    extern __shared__ __align__(16) unsigned char q2_smem[];
    T* us = reinterpret_cast<T*>(q2_smem);
    T* ws = us + 81 * BS;
    const int tid = threadIdx.x;
    const int64_t e = blockIdx.x * (int64_t)BS + tid;
    if (e >= g.n_el) return;
#pragma unroll 5
    for (int j = 0; j < 125; j++) q2_cp_async<sizeof(T)>(&ws[j * BS + tid], W + (int64_t)j * g.n_el + e);
    asm volatile("cp.async.commit_group;\n" ::: "memory");
    int ex[3];
    double h[3];
    q2e3(g, e, ex, h);
    const T sc[3] = {(T)2 / (T)h[0], (T)2 / (T)h[1], (T)2 / (T)h[2]};
    uint32_t fixbits[3] = {0u, 0u, 0u};   // bit A of word i: dof (A, i) is Dirichlet
#pragma unroll 1
    for (int A = 0; A < 27; A++) {
        const int64_t n = q2node3(g, ex, A);
#pragma unroll
        for (int c = 0; c < 3; c++) {
            const bool fx = bc[n * 3 + c] != 0;
            if (fx) fixbits[c] |= 1u << A;
            us[(A * 3 + c) * BS + tid] = (fx && mask_in) ? (T)0 : x[n * 3 + c];
        }
    }
    asm volatile("cp.async.wait_group 0;\n" ::: "memory");
    const T* Wp = ws + tid;
    q2_3d_apply_component<T, BS, 0>(g, us, Wp, BS, sc, ex, fixbits[0], y);
    q2_3d_apply_component<T, BS, 1>(g, us, Wp, BS, sc, ex, fixbits[1], y);
    q2_3d_apply_component<T, BS, 2>(g, us, Wp, BS, sc, ex, fixbits[2], y);
}

// ---------------------------------------------------------------------------
// FP64 apply from stored element matrices.  GB300 runs FP64 at 1/64 of the FP32
// rate, so the FP64 operator (the refinement residuals of the mixed solve and
// the plain FP64 solve) is applied from the 81x81 element matrices (symmetric,
// 3321 packed entries, element-major): 6561 FMAs per element instead of the
// ~25k of the matrix-free pass.  They are built once per assembly from the 125
// weights, sum-factorised:
//   K_(A,i),(B,j) = delta_ij sum_k M_kk(A,B) + M_ji(A,B),
//   M_kl(A,B) = sum_points w d_k N_A d_l N_B,
// each M_kl a separable contraction of the weights over x, then y, then z.
// ---------------------------------------------------------------------------
constexpr int KE_N = 81 * 82 / 2;   // 3321

__device__ __forceinline__ int ke_idx(int r, int c) {   // r <= c, row-major upper triangle
    return r * 81 - r * (r - 1) / 2 + (c - r);
}

// one warp per element; shared scratch per warp
struct ElmatScratch {
    double w[125];
    double T1[5 * 5 * 9];     // [q][r][ax*3+bx]
    double T2[5 * 81];        // [r][(ax*3+bx)*9 + ay*3+by]
    double M[729];            // [(ax,bx)][(ay,by)][(az,bz)]
    double L[729];
};

__global__ void __launch_bounds__(32) k_elmat_q2_3d(uwg_lgeom g, const double* __restrict__ W, double* Ke) {
    extern __shared__ double smem_raw[];
    ElmatScratch& S = *reinterpret_cast<ElmatScratch*>(smem_raw);
    const int lane = threadIdx.x;
    const int64_t e = blockIdx.x;
    if (e >= g.n_el) return;
    int ex[3];
    double h[3];
    q2e3(g, e, ex, h);
    const double sc[3] = {2.0 / h[0], 2.0 / h[1], 2.0 / h[2]};
    for (int j = lane; j < 125; j += 32) S.w[j] = W[(int64_t)j * g.n_el + e];
    for (int j = lane; j < 729; j += 32) S.L[j] = 0.0;
    double* out = Ke + e * (int64_t)KE_N;
    for (int j = lane; j < KE_N; j += 32) out[j] = 0.0;
    __syncwarp();
    for (int k = 0; k < 3; k++)
        for (int l = 0; l < 3; l++) {
            // axis factors: X (test side, derivative on axis k), Y (trial side, derivative on axis l)
            auto X = [&](int d, int t, int a) { return d == k ? sc[d] * c3_D5[t][a] : c3_B5[t][a]; };
            auto Y = [&](int d, int t, int b) { return d == l ? sc[d] * c3_D5[t][b] : c3_B5[t][b]; };
            for (int o = lane; o < 225; o += 32) {          // T1[q][r][ab_x]
                const int ab = o % 9, qr = o / 9, q = qr % 5, r = qr / 5;
                const int a = ab / 3, b = ab % 3;
                double s = 0.0;
                for (int p = 0; p < 5; p++) s += S.w[p + 5 * q + 25 * r] * (X(0, p, a) * Y(0, p, b));
                S.T1[(q + 5 * r) * 9 + ab] = s;
            }
            __syncwarp();
            for (int o = lane; o < 405; o += 32) {          // T2[r][abx][aby]
                const int aby = o % 9, abx = (o / 9) % 9, r = o / 81;
                const int a = aby / 3, b = aby % 3;
                double s = 0.0;
                for (int q = 0; q < 5; q++) s += S.T1[(q + 5 * r) * 9 + abx] * (X(1, q, a) * Y(1, q, b));
                S.T2[r * 81 + abx * 9 + aby] = s;
            }
            __syncwarp();
            for (int o = lane; o < 729; o += 32) {          // M[abx][aby][abz]
                const int abz = o % 9, xy = o / 9;
                const int a = abz / 3, b = abz % 3;
                double s = 0.0;
                for (int r = 0; r < 5; r++) s += S.T2[r * 81 + xy] * (X(2, r, a) * Y(2, r, b));
                S.M[o] = s;
            }
            __syncwarp();
            // M_kl(A, B) -> K[(A, l), (B, k)] (upper triangle); diagonal sums into L
            for (int o = lane; o < 729; o += 32) {
                const int abz = o % 9, aby = (o / 9) % 9, abx = o / 81;
                const int A = (abx / 3) + 3 * (aby / 3) + 9 * (abz / 3);
                const int B = (abx % 3) + 3 * (aby % 3) + 9 * (abz % 3);
                const double v = S.M[o];
                if (k == l) S.L[A * 27 + B] += v;
                const int rr = 3 * A + l, cc = 3 * B + k;
                if (rr <= cc) out[ke_idx(rr, cc)] += v;
            }
            __syncwarp();
        }
    for (int o = lane; o < 729; o += 32) {
        const int A = o / 27, B = o % 27;
        for (int i = 0; i < 3; i++) {
            const int rr = 3 * A + i, cc = 3 * B + i;
            if (rr <= cc) out[ke_idx(rr, cc)] += S.L[o];
        }
    }
}

// y += K x from the stored element matrices: one warp per element, lane owns rows
__global__ void __launch_bounds__(128) k_applyK_q2_3d_em(uwg_lgeom g, const double* __restrict__ Ke,
                                                         const uint8_t* __restrict__ bc, bool mask_in,
                                                         const double* __restrict__ x, double* y) {
    __shared__ double us[4][81];
    const int lane = threadIdx.x & 31, wl = threadIdx.x >> 5;
    const int64_t e = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    if (e >= g.n_el) return;   // warp-uniform
    int ex[3];
    double h[3];
    q2e3(g, e, ex, h);
    for (int k = lane; k < 81; k += 32) {
        const int64_t dof = q2node3(g, ex, k / 3) * 3 + k % 3;
        us[wl][k] = (mask_in && bc[dof]) ? 0.0 : x[dof];
    }
    __syncwarp();
    const double* K = Ke + e * (int64_t)KE_N;
    for (int rr = lane; rr < 81; rr += 32) {
        double s = 0.0;
        for (int cc = 0; cc < 81; cc++) s += K[rr <= cc ? ke_idx(rr, cc) : ke_idx(cc, rr)] * us[wl][cc];
        const int64_t dof = q2node3(g, ex, rr / 3) * 3 + rr % 3;
        if (!bc[dof]) atomicAdd(&y[dof], s);
    }
}

// ---------------------------------------------------------------------------
// Refinement residuals in double-float arithmetic.  The mixed solve's FP64
// refinement needs K x to a relative accuracy far below its 1e-8 target, not
// to the last FP64 bit, and GB300 runs FP64 at 1/64 of the FP32 rate.  Each
// element-matrix entry is stored as a pair of floats (hi, lo) with
// hi + lo = K to about 2^-48, each x value is split the same way, and a row is
// accumulated with the error-free transformations of Dekker (TwoProd, with
// FMA) and Knuth (TwoSum) on the FP32 pipes.  The plain FP64 solve, the
// right-hand side lifting and the reported residuals use the FP64 apply.
// ---------------------------------------------------------------------------
__global__ void k_split_df(int64_t n, const double* __restrict__ in, float2* __restrict__ out) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const double v = in[i];
        const float hi = (float)v;
        out[i] = make_float2(hi, (float)(v - (double)hi));
    }
}

// y += K x over free dofs from the double-float element matrices: one warp per
// element, lane owns rows (the layout of k_applyK_q2_3d_em)
__global__ void __launch_bounds__(128) k_applyK_q2_3d_df(uwg_lgeom g, const float2* __restrict__ Ke,
                                                         const uint8_t* __restrict__ bc,
                                                         const double* __restrict__ x, double* y) {
    __shared__ float2 us[4][81];
    const int lane = threadIdx.x & 31, wl = threadIdx.x >> 5;
    const int64_t e = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    if (e >= g.n_el) return;   // warp-uniform
    int ex[3];
    double h[3];
    q2e3(g, e, ex, h);
    for (int k = lane; k < 81; k += 32) {
        const int64_t dof = q2node3(g, ex, k / 3) * 3 + k % 3;
        const double v = bc[dof] ? 0.0 : x[dof];
        const float hi = (float)v;
        us[wl][k] = make_float2(hi, (float)(v - (double)hi));
    }
    __syncwarp();
    const float2* K = Ke + e * (int64_t)KE_N;
    for (int rr = lane; rr < 81; rr += 32) {
        float sh = 0.0f, sl = 0.0f;
        for (int cc = 0; cc < 81; cc++) {
            const float2 k = K[rr <= cc ? ke_idx(rr, cc) : ke_idx(cc, rr)];
            const float2 u = us[wl][cc];
            const float ph = k.x * u.x;                 // TwoProd: ph + pl = k.x u.x exactly
            float pl = fmaf(k.x, u.x, -ph);
            pl = fmaf(k.x, u.y, pl);                    // cross terms into the low part
            pl = fmaf(k.y, u.x, pl);
            const float s = sh + ph;                    // TwoSum: s + err = sh + ph exactly
            const float bb = s - sh;
            const float err = (sh - (s - bb)) + (ph - bb);
            sh = s;
            sl += err + pl;
        }
        const int64_t dof = q2node3(g, ex, rr / 3) * 3 + rr % 3;
        if (!bc[dof]) atomicAdd(&y[dof], (double)sh + (double)sl);
    }
}

// G_e[(A,i)][k] = -(prod_{j != i} h_j / 2) GR[i][A][k]
__device__ __forceinline__ double q2_Ge3(const double* h, int A, int i, int k) {
    const double f = i == 0 ? (h[1] * 0.5) * (h[2] * 0.5) : (i == 1 ? (h[0] * 0.5) * (h[2] * 0.5) : (h[0] * 0.5) * (h[1] * 0.5));
    return -f * c3_GR[i][A][k];
}

// Diagonal of K (assembled over free dofs) and, per element, the inverse of S^_e.
// diag K_(A,i) = sum_points w (|grad N_A|^2 + (d_i N_A)^2); each of the three
// squared-derivative sums is a separable contraction of the 125 weights.
__global__ void k_diag_q2_3d(uwg_lgeom g, const double* W, const uint8_t* bc, double* diag, double* sinv) {
    int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (e >= g.n_el) return;
    int ex[3];
    double h[3];
    q2e3(g, e, ex, h);
    const double s2[3] = {4.0 / (h[0] * h[0]), 4.0 / (h[1] * h[1]), 4.0 / (h[2] * h[2])};
    double kd[27][3];
    for (int A = 0; A < 27; A++) kd[A][0] = kd[A][1] = kd[A][2] = 0.0;
    // Dj[A] = sum_points w (d_j N_A / s_j)^2 for j = 0, 1, 2
    double Dsum[3][27];
    for (int j = 0; j < 3; j++)
        for (int A = 0; A < 27; A++) Dsum[j][A] = 0.0;
    for (int r = 0; r < 5; r++)
        for (int q = 0; q < 5; q++)
            for (int p = 0; p < 5; p++) {
                const double w = W[(int64_t)(p + 5 * q + 25 * r) * g.n_el + e];
                for (int A = 0; A < 27; A++) {
                    const int a = A % 3, b = (A / 3) % 3, c = A / 9;
                    const double bx = c3_B5[p][a], by = c3_B5[q][b], bz = c3_B5[r][c];
                    const double dx = c3_D5[p][a] * by * bz, dy = bx * c3_D5[q][b] * bz, dz = bx * by * c3_D5[r][c];
                    Dsum[0][A] += w * dx * dx;
                    Dsum[1][A] += w * dy * dy;
                    Dsum[2][A] += w * dz * dz;
                }
            }
    for (int A = 0; A < 27; A++) {
        const double gsq = s2[0] * Dsum[0][A] + s2[1] * Dsum[1][A] + s2[2] * Dsum[2][A];
        for (int i = 0; i < 3; i++) kd[A][i] = gsq + s2[i] * Dsum[i][A];
    }
    for (int A = 0; A < 27; A++) {
        const int64_t n = q2node3(g, ex, A);
        for (int i = 0; i < 3; i++)
            if (!bc[n * 3 + i]) atomicAdd(&diag[n * 3 + i], kd[A][i]);
    }
    if (!sinv) return;
    double S[4][8];
    for (int k = 0; k < 4; k++)
        for (int l = 0; l < 4; l++) {
            double s = 0.0;
            for (int A = 0; A < 27; A++)
                for (int i = 0; i < 3; i++) s += q2_Ge3(h, A, i, k) * (q2_Ge3(h, A, i, l) / kd[A][i]);
            S[k][l] = s;
            S[k][4 + l] = k == l ? 1.0 : 0.0;
        }
    // Gauss-Jordan with partial pivoting on the 4x4 block
    for (int col = 0; col < 4; col++) {
        int piv = col;
        for (int r = col + 1; r < 4; r++)
            if (fabs(S[r][col]) > fabs(S[piv][col])) piv = r;
        if (piv != col)
            for (int k = 0; k < 8; k++) { double t = S[col][k]; S[col][k] = S[piv][k]; S[piv][k] = t; }
        const double d = 1.0 / S[col][col];
        for (int k = 0; k < 8; k++) S[col][k] *= d;
        for (int r = 0; r < 4; r++) {
            if (r == col) continue;
            const double f = S[r][col];
            for (int k = 0; k < 8; k++) S[r][k] -= f * S[col][k];
        }
    }
    double* o = sinv + e * 16;
    for (int k = 0; k < 4; k++)
        for (int l = 0; l < 4; l++) o[k * 4 + l] = S[k][4 + l];
}

__global__ void k_applyG_q2_3d(uwg_lgeom g, const uint8_t* bc, const double* p, double* y) {
    int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (e >= g.n_el) return;
    int ex[3];
    double h[3];
    q2e3(g, e, ex, h);
    const double pe[4] = {p[e * 4], p[e * 4 + 1], p[e * 4 + 2], p[e * 4 + 3]};
    for (int A = 0; A < 27; A++) {
        const int64_t n = q2node3(g, ex, A);
        for (int i = 0; i < 3; i++) {
            if (bc[n * 3 + i]) continue;
            double s = 0.0;
            for (int k = 0; k < 4; k++) s += q2_Ge3(h, A, i, k) * pe[k];
            atomicAdd(&y[n * 3 + i], s);
        }
    }
}

__global__ void k_applyGt_q2_3d(uwg_lgeom g, const uint8_t* bc, int only_bc, const double* u, double* q) {
    int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (e >= g.n_el) return;
    int ex[3];
    double h[3];
    q2e3(g, e, ex, h);
    double s[4] = {0.0, 0.0, 0.0, 0.0};
    for (int A = 0; A < 27; A++) {
        const int64_t n = q2node3(g, ex, A);
        for (int i = 0; i < 3; i++) {
            if ((bc[n * 3 + i] != 0) != (only_bc != 0)) continue;
            const double v = u[n * 3 + i];
            for (int k = 0; k < 4; k++) s[k] += q2_Ge3(h, A, i, k) * v;
        }
    }
    for (int k = 0; k < 4; k++) q[e * 4 + k] = s[k];
}

__global__ void k_schur_pc_q2_3d(int64_t n_el, const double* sinv, const double* r, double* z) {
    int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (e >= n_el) return;
    const double* S = sinv + e * 16;
    const double r0 = r[e * 4], r1 = r[e * 4 + 1], r2 = r[e * 4 + 2], r3 = r[e * 4 + 3];
    for (int k = 0; k < 4; k++) z[e * 4 + k] = S[4 * k] * r0 + S[4 * k + 1] * r1 + S[4 * k + 2] * r2 + S[4 * k + 3] * r3;
}

// Element matrices of one element (diagnostics): K_e from the 125 weights by
// the direct formula K_(A,i),(B,j) = sum_points w (delta_ij grad N_A . grad N_B
// + d_j N_A d_i N_B), G_e and S^_e.  One block of 81 threads, thread = column.
__global__ void k_element_matrices_q2_3d(uwg_lgeom g, int64_t e, const double* W, double* Ke, double* Ge_out,
                                         double* Se) {
    int ex[3];
    double h[3];
    q2e3(g, e, ex, h);
    const double s[3] = {2.0 / h[0], 2.0 / h[1], 2.0 / h[2]};
    const int col = threadIdx.x;
    if (col < 81) {
        const int B = col / 3, j = col % 3;
        const int ba = B % 3, bb = (B / 3) % 3, bc_ = B / 9;
        double acc[81];
        for (int k = 0; k < 81; k++) acc[k] = 0.0;
        for (int r = 0; r < 5; r++)
            for (int q = 0; q < 5; q++)
                for (int p = 0; p < 5; p++) {
                    const double w = W[(int64_t)(p + 5 * q + 25 * r) * g.n_el + e];
                    const double gB[3] = {s[0] * c3_D5[p][ba] * c3_B5[q][bb] * c3_B5[r][bc_],
                                          s[1] * c3_B5[p][ba] * c3_D5[q][bb] * c3_B5[r][bc_],
                                          s[2] * c3_B5[p][ba] * c3_B5[q][bb] * c3_D5[r][bc_]};
                    for (int A = 0; A < 27; A++) {
                        const int a = A % 3, b = (A / 3) % 3, c = A / 9;
                        const double gA[3] = {s[0] * c3_D5[p][a] * c3_B5[q][b] * c3_B5[r][c],
                                              s[1] * c3_B5[p][a] * c3_D5[q][b] * c3_B5[r][c],
                                              s[2] * c3_B5[p][a] * c3_B5[q][b] * c3_D5[r][c]};
                        const double dot = gA[0] * gB[0] + gA[1] * gB[1] + gA[2] * gB[2];
                        for (int i = 0; i < 3; i++) acc[A * 3 + i] += w * ((i == j ? dot : 0.0) + gA[j] * gB[i]);
                    }
                }
        for (int k = 0; k < 81; k++) Ke[k * 81 + col] = acc[k];
        for (int k = 0; k < 4; k++) Ge_out[col * 4 + k] = q2_Ge3(h, B, j, k);
    }
    __syncthreads();
    if (col < 16) {
        const int k = col / 4, l = col % 4;
        double sum = 0.0;
        for (int rr = 0; rr < 81; rr++) sum += Ge_out[rr * 4 + k] * (Ge_out[rr * 4 + l] / Ke[rr * 81 + rr]);
        Se[k * 4 + l] = sum;
    }
}

void dpc1_3d_host(double xi, double eta, double zeta, double* M) {
    const double fac = 1.0 / 9.0;
    M[0] = fac * (-4.0 * xi - 20.0 * eta + 12.0 * zeta + 3.0);
    M[1] = fac * (16.0 * xi - 64.0 * eta + 60.0 * zeta + 6.0);
    M[2] = fac * (36.0 * eta - 36.0 * zeta);
    M[3] = fac * (-12.0 * xi + 48.0 * eta - 36.0 * zeta);
}
void q2_1d_host3(double s, double* N, double* D) {
    N[0] = 0.5 * s * (s - 1.0); N[1] = 1.0 - s * s; N[2] = 0.5 * s * (s + 1.0);
    D[0] = s - 0.5; D[1] = -2.0 * s; D[2] = s + 0.5;
}

}  // namespace

// ---------------------------------------------------------------------------
// Host wrappers (called by the uwg_q2_* dispatchers for 3D contexts)
// ---------------------------------------------------------------------------
int uwg_q2_3d_init(uwg_ctx* c) {
    // reference gradient integrals, 3-point Gauss (exact: degree <= 3 per axis)
    const double gp[3] = {-std::sqrt(0.6), 0.0, std::sqrt(0.6)}, gw[3] = {5.0 / 9.0, 8.0 / 9.0, 5.0 / 9.0};
    static double GR[3][27][4];
    for (int i = 0; i < 3; i++)
        for (int A = 0; A < 27; A++)
            for (int k = 0; k < 4; k++) GR[i][A][k] = 0.0;
    for (int kz = 0; kz < 3; kz++)
        for (int jy = 0; jy < 3; jy++)
            for (int ix = 0; ix < 3; ix++) {
                double Nx[3], Dx[3], Ny[3], Dy[3], Nz[3], Dz[3], M[4];
                q2_1d_host3(gp[ix], Nx, Dx);
                q2_1d_host3(gp[jy], Ny, Dy);
                q2_1d_host3(gp[kz], Nz, Dz);
                dpc1_3d_host(gp[ix], gp[jy], gp[kz], M);
                const double w = gw[ix] * gw[jy] * gw[kz];
                for (int A = 0; A < 27; A++) {
                    const int a = A % 3, b = (A / 3) % 3, cc = A / 9;
                    for (int k = 0; k < 4; k++) {
                        GR[0][A][k] += w * Dx[a] * Ny[b] * Nz[cc] * M[k];
                        GR[1][A][k] += w * Nx[a] * Dy[b] * Nz[cc] * M[k];
                        GR[2][A][k] += w * Nx[a] * Ny[b] * Dz[cc] * M[k];
                    }
                }
            }
    UWG_CUDA(c, cudaMemcpyToSymbol(c3_GR, GR, sizeof(GR)));
    return UWG_OK;
}

int uwg_q2_3d_assemble(uwg_ctx* c, const int32_t* off, const int32_t* list, const double* ip_xi, const double* ip_w,
                       const double* eta_p, const double* body_p) {
    uwg_lgeom g = uwg_level_geom(c, 0);
    // the applies stage 105 KB per block (set here, before any solve is captured)
    UWG_CUDA(c, cudaFuncSetAttribute(k_applyK_q2_3d<float, 128>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)q2_3d_apply_smem<float, 128>()));
    UWG_CUDA(c, cudaFuncSetAttribute(k_applyK_q2_3d<double, 64>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)q2_3d_apply_smem<double, 64>()));
    vk_zero<double>(c->stream, c->n_vdof, c->f);
    k_assemble_q2_3d<<<nblk(c->n_el * 32, 128), 128, 0, c->stream>>>(g, off, list, ip_xi, ip_w, eta_p, body_p,
                                                                    c->lev[0].W64, c->lev[1].W64, c->f);
    UWG_CUDA(c, cudaGetLastError());
    // element matrices of the FP64 apply, rebuilt with every assembly (before the
    // right-hand side's Dirichlet lifting uses the operator)
    if (!c->q2_ke) {
        cudaError_t e = cudaMalloc((void**)&c->q2_ke, sizeof(double) * (size_t)KE_N * c->n_el);
        if (e != cudaSuccess) {
            c->q2_ke = nullptr;   // no room: the matrix-free FP64 apply is used
            cudaGetLastError();
        }
    }
    if (c->q2_ke) {
        k_elmat_q2_3d<<<(unsigned)c->n_el, 32, sizeof(ElmatScratch), c->stream>>>(g, c->lev[0].W64, c->q2_ke);
        UWG_CUDA(c, cudaGetLastError());
        if (!c->q2_ke_df) {
            cudaError_t e = cudaMalloc((void**)&c->q2_ke_df, sizeof(float2) * (size_t)KE_N * c->n_el);
            if (e != cudaSuccess) {
                c->q2_ke_df = nullptr;   // no room: refinement residuals use the FP64 apply
                cudaGetLastError();
            }
        }
        if (c->q2_ke_df) {
            k_split_df<<<152 * 16, 256, 0, c->stream>>>((int64_t)KE_N * c->n_el, c->q2_ke, c->q2_ke_df);
            UWG_CUDA(c, cudaGetLastError());
        }
    }
    return UWG_OK;
}

template <typename T>
int uwg_q2_3d_applyK(uwg_ctx* c, const T* x, T* y, bool mask_in) {
    const uwg_level& L = c->lev[0];
    if constexpr (sizeof(T) == 8) {
        if (c->q2_ke) {
            k_applyK_q2_3d_em<<<nblk(L.n_el * 32, 128), 128, 0, c->stream>>>(uwg_level_geom(c, 0), c->q2_ke, L.bc,
                                                                             mask_in, x, y);
            UWG_CUDA(c, cudaGetLastError());
            return UWG_OK;
        }
    }
    const T* W;
    if constexpr (sizeof(T) == 8) W = (const T*)L.W64; else W = (const T*)L.W32;
    constexpr int BS = sizeof(T) == 8 ? 64 : 128;
    k_applyK_q2_3d<T, BS><<<nblk(L.n_el, BS), BS, q2_3d_apply_smem<T, BS>(), c->stream>>>(uwg_level_geom(c, 0), W,
                                                                                         L.bc, mask_in, x, y);
    UWG_CUDA(c, cudaGetLastError());
    return UWG_OK;
}
template int uwg_q2_3d_applyK<double>(uwg_ctx*, const double*, double*, bool);

// y += K x at free dofs in double-float arithmetic; UWG_ERR_STATE when the
// double-float element matrices are absent (the caller then uses the FP64 apply)
int uwg_q2_3d_applyK_df(uwg_ctx* c, const double* x, double* y) {
    if (!c->q2_ke_df) return UWG_ERR_STATE;
    const uwg_level& L = c->lev[0];
    k_applyK_q2_3d_df<<<nblk(L.n_el * 32, 128), 128, 0, c->stream>>>(uwg_level_geom(c, 0), c->q2_ke_df, L.bc, x, y);
    UWG_CUDA(c, cudaGetLastError());
    return UWG_OK;
}
template int uwg_q2_3d_applyK<float>(uwg_ctx*, const float*, float*, bool);

int uwg_q2_3d_diag(uwg_ctx* c, double* sinv) {
    const uwg_level& L = c->lev[0];

    k_diag_q2_3d<<<nblk(L.n_el, 64), 64, 0, c->stream>>>(uwg_level_geom(c, 0), L.W64, L.bc, L.diag64, sinv);
    UWG_CUDA(c, cudaGetLastError());
    return UWG_OK;
}

int uwg_q2_3d_applyG(uwg_ctx* c, const double* p, double* y) {
    vk_zero<double>(c->stream, c->n_vdof, y);
    k_applyG_q2_3d<<<nblk(c->n_el), 256, 0, c->stream>>>(uwg_level_geom(c, 0), c->bc, p, y);
    UWG_CUDA(c, cudaGetLastError());
    return UWG_OK;
}

int uwg_q2_3d_applyGt(uwg_ctx* c, const double* u, double* q, int only_bc) {
    k_applyGt_q2_3d<<<nblk(c->n_el), 256, 0, c->stream>>>(uwg_level_geom(c, 0), c->bc, only_bc, u, q);
    UWG_CUDA(c, cudaGetLastError());
    return UWG_OK;
}

int uwg_q2_3d_schur_pc(uwg_ctx* c, const double* r, double* z) {
    k_schur_pc_q2_3d<<<nblk(c->n_el), 256, 0, c->stream>>>(c->n_el, c->Shat, r, z);
    UWG_CUDA(c, cudaGetLastError());
    return UWG_OK;
}

int uwg_q2_3d_element_matrices(uwg_ctx* c, int64_t el, double* Ke, double* Ge, double* Se) {
    double* buf = nullptr;
    const int nk = 81 * 81, ng = 81 * 4, ns = 16;
    UWG_CUDA(c, cudaMallocAsync((void**)&buf, sizeof(double) * (nk + ng + ns), c->stream));
    k_element_matrices_q2_3d<<<1, 96, 0, c->stream>>>(uwg_level_geom(c, 0), el, c->lev[0].W64, buf, buf + nk,
                                                      buf + nk + ng);
    std::vector<double> h(nk + ng + ns);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaMemcpyAsync(h.data(), buf, sizeof(double) * h.size(), cudaMemcpyDeviceToHost, c->stream);
    cudaFreeAsync(buf, c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) return uwg_set_error(c, UWG_ERR_CUDA, cudaGetErrorString(e));
    if (Ke) for (int i = 0; i < nk; i++) Ke[i] = h[i];
    if (Ge) for (int i = 0; i < ng; i++) Ge[i] = h[nk + i];
    if (Se) for (int i = 0; i < ns; i++) Se[i] = h[nk + ng + i];
    return UWG_OK;
}
