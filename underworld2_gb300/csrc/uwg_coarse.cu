// Coarse-level correction of the Schur-complement flexible GMRES (2D Q1/dQ0).
// No counterpart in the reference, whose BSSCR preconditions the Schur
// complement with one operator (L/Solvers/KSPSolvers/src/BSSCR/bsscr.c).
//
// Pressure cells are aggregated in agg x agg blocks (P: piecewise-constant
// prolongation).  The coarse Schur complement is the Galerkin product on a
// coarse velocity space: Sc = Gc^T Kc^-1 Gc with Kc the velocity multigrid's
// Galerkin operator on the level whose elements are agg / 2 fine cells wide
// (2 x 2 coarse elements per aggregate) and Gc = I^T G P, which for nested
// bilinear velocity spaces is the coarse mesh's own divergence integrated over
// each aggregate: Gc[A, J] = -int_{aggregate J} d N_A / d x_i.
//
// Kc is banded (node-major dofs on a structured grid: half-bandwidth
// dim (nodes per row + 1) + dim - 1), so it is factored by a banded Cholesky
// in one CTA with the active (b+1) x (b+1) window in shared memory; then
// Y = L^-1 Gc (FP32 forward substitution, one warp per aggregate), Sc = Y^T Y,
// and Sc^-1 densely (the constant mode fixed by a rank-one term when the
// constant pressure is in the null space of G).
//
// Each preconditioner application (right-preconditioned FGMRES on A = -S):
//   y = BFBt(r), s = A y (one extra Schur apply, loose velocity tolerance),
//   z = y + Q (r - s),  Q = P (P^T A P)^-1 P^T = -P Sc^-1 P^T,
// the deflation step of the two-level "A-DEF2" preconditioner (Tang, Nabben,
// Vuik & Erlangga, J. Sci. Comput. 39, 2009).
#include <cmath>
#include <cstring>
#include <vector>

#include "uwg_internal.cuh"
#include "uwg_ops.cuh"

namespace {

__global__ void k_band_extract(int64_t n, int b, const double* __restrict__ A, double* __restrict__ Ab) {
    const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (t >= n * (b + 1)) return;
    const int64_t j = t / (b + 1);
    const int d = (int)(t % (b + 1));
    Ab[t] = (j + d < n) ? A[(j + d) * n + j] : 0.0;
}

// Ab[j * (b+1) + d] = A[j + d][j] on entry, L[j + d][j] on exit (A = L L^T).
// Slot (j mod (b+1)) of the shared window holds column j of the band while
// j is in [k, k + b].  Step k, with a = column k:
//   A  threads d <= b: sc[d] = a_d / a_kk, L[k+d][k] = a_d / sqrt(a_kk) to
//      global (one reciprocal and square root per warp, shuffled);
//   B  all threads: A[k+i][k+j] -= sc[i] a_j for 1 <= j <= i <= m;
//   C  threads d <= b: the slot of column k takes column k + b + 1, whose
//      global load was issued at the start of the step (no earlier step
//      touches that column).
// FP64 throughput of one SM bounds it, hence one division per warp rather
// than per thread.  A non-positive pivot sets bit 0 of *status.
__global__ void __launch_bounds__(1024) k_band_cholesky(int n, int b, double* __restrict__ Ab, int* status) {
    extern __shared__ double win[];   // [(b+1)][(b+1)] window, then sc[b+1]
    const int B1 = b + 1, tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
    double* sc = win + B1 * B1;
    for (int t = threadIdx.x; t < B1 * B1; t += blockDim.x) {
        const int j = t / B1, d = t - j * B1;
        win[t] = j < n ? Ab[(int64_t)j * B1 + d] : 0.0;
    }
    __syncthreads();
    const int d = threadIdx.x;
    const bool colw = ty <= (B1 - 1) / 32;   // warps holding the threads d <= b
    for (int k = 0; k < n; k++) {
        const int sk = k % B1;
        double* ck = win + sk * B1;
        const int m = min(b, n - 1 - k);
        double next = 0.0;
        if (colw) {
            if (d < B1 && k + B1 < n) next = Ab[(int64_t)(k + B1) * B1 + d];
            double inv = 0.0, rs = 0.0;
            if (tx == 0) {
                double akk = ck[0];
                if (!(akk > 0.0)) {
                    if (ty == 0) atomicOr(status, 1);
                    akk = 1.0;
                }
                inv = 1.0 / akk;
                rs = inv * sqrt(akk);   // 1 / sqrt(a_kk)
            }
            inv = __shfl_sync(0xffffffffu, inv, 0);
            rs = __shfl_sync(0xffffffffu, rs, 0);
            if (d < B1) {
                const double a = ck[d];
                sc[d] = a * inv;
                Ab[(int64_t)k * B1 + d] = a * rs;   // d = 0: a_kk / sqrt(a_kk)
            }
        }
        __syncthreads();
        for (int i0 = 0; i0 < m; i0 += 32) {
            const int di = i0 + ty + 1;
            if (di > m) break;
            const double si = sc[di];
            for (int j0 = 0; j0 <= i0; j0 += 32) {
                const int dj = j0 + tx + 1;
                if (dj > di) continue;
                int slot = sk + dj;
                if (slot >= B1) slot -= B1;
                win[slot * B1 + (di - dj)] -= si * ck[dj];
            }
        }
        __syncthreads();
        if (colw && d < B1) ck[d] = next;
    }
}

// Y = L^-1 G in FP32 (L converted from the FP64 factor), G and Y row-major
// [n][nrhs]; one warp per right-hand side, the last b values of its solution
// in a shared circular buffer; two warps per CTA so that the right-hand sides
// spread over many SMs.  Y only shapes the preconditioner of a flexible
// GMRES: its FP32 error (about cond(L) x 6e-8) changes iteration counts, not
// results; FP64 would be bound by the FP64 pipe.
__global__ void __launch_bounds__(64) k_band_forward(int n, int b, int nrhs, const float* __restrict__ Lb,
                                                     const double* __restrict__ G, float* __restrict__ Y) {
    extern __shared__ float yb[];   // [2 warps][b + 1]
    const int lane = threadIdx.x & 31, wl = threadIdx.x >> 5;
    const int j = blockIdx.x * 2 + wl;
    if (j >= nrhs) return;
    const int B1 = b + 1;
    float* buf = yb + wl * B1;
    for (int k = 0; k < n; k++) {
        const int dm = min(b, k);
        float s = 0.f;
        for (int d = lane + 1; d <= dm; d += 32) {
            int slot = k - d;
            slot -= (slot / B1) * B1;
            s = fmaf(Lb[(int64_t)(k - d) * B1 + d], buf[slot], s);
        }
        for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
        if (lane == 0) {
            const float y = ((float)G[(int64_t)k * nrhs + j] - s) / Lb[(int64_t)k * B1];
            buf[k % B1] = y;
            Y[(int64_t)k * nrhs + j] = y;
        }
        __syncwarp();
    }
}

__global__ void k_d2f(int64_t n, const double* __restrict__ a, float* __restrict__ b) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i < n) b[i] = (float)a[i];
}

// C = Y^T Y (FP64 sums of FP32 entries), Y row-major [n][m], C [m][m]; 16 x 16 tiles.
__global__ void k_gram(int n, int m, const float* __restrict__ Y, double* __restrict__ C) {
    __shared__ double As[16][17], Bs[16][17];
    const int tx = threadIdx.x, ty = threadIdx.y;
    const int i = blockIdx.y * 16 + ty, j = blockIdx.x * 16 + tx;
    double acc = 0.0;
    for (int k0 = 0; k0 < n; k0 += 16) {
        const int k = k0 + ty;
        const int ia = blockIdx.y * 16 + tx;
        As[ty][tx] = (k < n && ia < m) ? (double)Y[(int64_t)k * m + ia] : 0.0;   // As[k][i]
        Bs[ty][tx] = (k < n && j < m) ? (double)Y[(int64_t)k * m + j] : 0.0;     // Bs[k][j]
        __syncthreads();
#pragma unroll
        for (int kk = 0; kk < 16; kk++) acc += As[kk][ty] * Bs[kk][tx];
        __syncthreads();
    }
    if (i < m && j < m) C[(int64_t)i * m + j] = acc;
}

// tc[J] = sum over the cells of aggregate J of (r - s); one warp per aggregate
__global__ void k_cc_restrict(int res0, int agg, int ncx, int npc, const double* __restrict__ r,
                              const double* __restrict__ s, double* __restrict__ tc) {
    const int J = (int)((blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5), lane = threadIdx.x & 31;
    if (J >= npc) return;
    const int cx0 = (J % ncx) * agg, cy0 = (J / ncx) * agg;
    double v = 0.0;
    for (int k = lane; k < agg * agg; k += 32) {
        const int64_t i = (cx0 + k % agg) + (int64_t)res0 * (cy0 + k / agg);
        v += r[i] - s[i];
    }
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if (lane == 0) tc[J] = v;
}

// zc = Sinv tc; one warp per row
__global__ void k_cc_mv(int npc, const double* __restrict__ Sinv, const double* __restrict__ tc,
                        double* __restrict__ zc) {
    const int i = (int)((blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5), lane = threadIdx.x & 31;
    if (i >= npc) return;
    double v = 0.0;
    for (int j = lane; j < npc; j += 32) v += Sinv[(int64_t)i * npc + j] * tc[j];
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if (lane == 0) zc[i] = v;
}

// z[i] -= zc[aggregate of cell i]
__global__ void k_cc_prolong_sub(int64_t np, int res0, int agg, int ncx, const double* __restrict__ zc,
                                 double* __restrict__ z) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= np) return;
    const int cx = (int)(i % res0), cy = (int)(i / res0);
    z[i] -= zc[(cx / agg) + ncx * (cy / agg)];
}

unsigned nb(int64_t n, int t = 256) { return (unsigned)((n + t - 1) / t); }

}  // namespace

int uwg_cc_dims(const uwg_ctx* c, int agg, int* npc, int* lv) {
    if (c->dim != 2 || c->order != 1 || c->porder != 0) return -1;
    if (agg < 2 || agg % 2 || c->res[0] % agg || c->res[1] % agg) return -2;
    const int ncx = c->res[0] / agg, ncy = c->res[1] / agg;
    *npc = ncx * ncy;
    *lv = -1;
    for (int l = 0; l < c->nlev; l++)
        if (c->lev[l].res[0] == 2 * ncx && c->lev[l].res[1] == 2 * ncy) *lv = l;
    return *lv < 0 ? -3 : 0;
}

int uwg_cc_build(uwg_ctx* c, int agg, bool const_null, double* sinv) {
    int npc = 0, lv = -1;
    const int dr = uwg_cc_dims(c, agg, &npc, &lv);
    if (dr == -1) return uwg_set_error(c, UWG_ERR_ARG, "coarse correction: 2D Q1/dQ0 only");
    if (dr == -2) return uwg_set_error(c, UWG_ERR_ARG, "coarse_agg must be even and divide the mesh resolution");
    if (dr == -3)
        return uwg_set_error(c, UWG_ERR_ARG, "coarse correction: no velocity multigrid level with elements "
                                             "coarse_agg / 2 fine cells wide");
    if (npc > 1024) return uwg_set_error(c, UWG_ERR_ARG, "coarse correction: more than 1024 aggregates");
    const uwg_level& L = c->lev[lv];
    const int64_t n = L.n_dof;
    const int nxn = L.res[0] + 1;
    const int b = 2 * (nxn + 1) + 1;   // half-bandwidth of node-major 2D Q1 dofs
    if (n > 20000 || b > 120)
        return uwg_set_error(c, UWG_ERR_ARG, "coarse correction: coarse velocity level too large");
    cudaStream_t s = c->stream;
    const int ncx = c->res[0] / agg;
    // Gc on the host from the coarse level's geometry and Dirichlet mask
    uwg_lgeom g = uwg_level_geom(c, lv);
    std::vector<double> ax0(L.res[0] + 1), ax1(L.res[1] + 1);
    std::vector<uint8_t> bch(n);
    UWG_CUDA(c, cudaMemcpyAsync(ax0.data(), g.ax[0], sizeof(double) * ax0.size(), cudaMemcpyDeviceToHost, s));
    UWG_CUDA(c, cudaMemcpyAsync(ax1.data(), g.ax[1], sizeof(double) * ax1.size(), cudaMemcpyDeviceToHost, s));
    UWG_CUDA(c, cudaMemcpyAsync(bch.data(), L.bc, n, cudaMemcpyDeviceToHost, s));
    UWG_CUDA(c, cudaStreamSynchronize(s));
    std::vector<double> Gh((size_t)n * npc, 0.0);
    for (int ey = 0; ey < L.res[1]; ey++)
        for (int ex = 0; ex < L.res[0]; ex++) {
            const double hx = ax0[ex + 1] - ax0[ex], hy = ax1[ey + 1] - ax1[ey];
            const int J = ex / 2 + ncx * (ey / 2);
            for (int a = 0; a < 4; a++) {
                const int64_t node = (ex + (a & 1)) + (int64_t)nxn * (ey + (a >> 1));
                for (int i = 0; i < 2; i++) {
                    // -int_e dN_a/dx_i = -(+-1) h_other / 2 (+ for the node on the high side of axis i)
                    const double v = (((a >> i) & 1) ? -0.5 : 0.5) * (i == 0 ? hy : hx);
                    const int64_t dof = node * 2 + i;
                    if (!bch[dof]) Gh[(size_t)dof * npc + J] += v;
                }
            }
        }
    double *A = nullptr, *Ab = nullptr, *G = nullptr, *Sc = nullptr, *Sc2 = nullptr;
    float *Y = nullptr, *Lf = nullptr;
    int* st = nullptr;
    auto cleanup = [&]() {
        for (void* p : {(void*)A, (void*)Ab, (void*)G, (void*)Y, (void*)Lf, (void*)Sc, (void*)Sc2, (void*)st})
            if (p) cudaFreeAsync(p, s);
    };
#define CC_TRY(call)                                                                                     \
    do {                                                                                                 \
        cudaError_t e_ = (call);                                                                         \
        if (e_ != cudaSuccess) {                                                                         \
            cleanup();                                                                                   \
            return uwg_set_error(c, UWG_ERR_CUDA, std::string("coarse correction: ") + cudaGetErrorString(e_)); \
        }                                                                                                \
    } while (0)
    CC_TRY(cudaMallocAsync((void**)&A, sizeof(double) * n * n, s));
    CC_TRY(cudaMallocAsync((void**)&Ab, sizeof(double) * n * (b + 1), s));
    CC_TRY(cudaMallocAsync((void**)&G, sizeof(double) * n * npc, s));
    CC_TRY(cudaMallocAsync((void**)&Y, sizeof(float) * n * npc, s));
    CC_TRY(cudaMallocAsync((void**)&Lf, sizeof(float) * n * (b + 1), s));
    CC_TRY(cudaMallocAsync((void**)&Sc, sizeof(double) * npc * npc, s));
    CC_TRY(cudaMallocAsync((void**)&Sc2, sizeof(double) * npc * npc, s));
    CC_TRY(cudaMallocAsync((void**)&st, sizeof(int), s));
    CC_TRY(cudaMemsetAsync(st, 0, sizeof(int), s));
    int rc = uwg_ops_dense_matrix(c, lv, A);
    if (rc) { cleanup(); return rc; }
    k_band_extract<<<nb(n * (b + 1)), 256, 0, s>>>(n, b, A, Ab);
    const size_t win = sizeof(double) * (b + 2) * (b + 1);
    CC_TRY(cudaFuncSetAttribute(k_band_cholesky, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)win));
    k_band_cholesky<<<1, 1024, win, s>>>((int)n, b, Ab, st);
    CC_TRY(cudaGetLastError());
    CC_TRY(cudaMemcpyAsync(G, Gh.data(), sizeof(double) * n * npc, cudaMemcpyHostToDevice, s));
    k_d2f<<<nb(n * (b + 1)), 256, 0, s>>>(n * (b + 1), Ab, Lf);
    k_band_forward<<<nb(npc, 2), 64, sizeof(float) * 2 * (b + 1), s>>>((int)n, b, npc, Lf, G, Y);
    k_gram<<<dim3(nb(npc, 16), nb(npc, 16)), dim3(16, 16), 0, s>>>((int)n, npc, Y, Sc);
    CC_TRY(cudaGetLastError());
    std::vector<double> Sh((size_t)npc * npc);
    int sth = 0;
    CC_TRY(cudaMemcpyAsync(Sh.data(), Sc, sizeof(double) * npc * npc, cudaMemcpyDeviceToHost, s));
    CC_TRY(cudaMemcpyAsync(&sth, st, sizeof(int), cudaMemcpyDeviceToHost, s));
    CC_TRY(cudaStreamSynchronize(s));   // Gh and Sh must outlive their copies
    if (sth) {
        cleanup();
        return uwg_set_error(c, UWG_ERR_NAN, "coarse correction: the coarse velocity operator is not positive definite");
    }
    double tr = 0.0;
    for (int i = 0; i < npc; i++) tr += Sh[(size_t)i * npc + i];
    const double fix = const_null ? tr / ((double)npc * npc) : 0.0;
    for (int i = 0; i < npc; i++)
        for (int j = 0; j < i; j++) {
            const double v = 0.5 * (Sh[(size_t)i * npc + j] + Sh[(size_t)j * npc + i]) + fix;
            Sh[(size_t)i * npc + j] = Sh[(size_t)j * npc + i] = v;
        }
    for (int i = 0; i < npc; i++) Sh[(size_t)i * npc + i] += fix;
    CC_TRY(cudaMemcpyAsync(Sc2, Sh.data(), sizeof(double) * npc * npc, cudaMemcpyHostToDevice, s));
    rc = uwg_ops_dense_invert_grid(c, npc, Sc2, sinv);
    if (rc) { cleanup(); return rc; }
    CC_TRY(cudaStreamSynchronize(s));   // Sh must outlive its copy
    cleanup();
#undef CC_TRY
    return UWG_OK;
}

int uwg_cc_apply(uwg_ctx* c, int agg, const double* sinv, double* tc, double* zc, const double* r, const double* sv,
                 double* z) {
    const int ncx = c->res[0] / agg, npc = ncx * (c->res[1] / agg);
    cudaStream_t s = c->stream;
    k_cc_restrict<<<nb((int64_t)npc * 32), 256, 0, s>>>(c->res[0], agg, ncx, npc, r, sv, tc);
    k_cc_mv<<<nb((int64_t)npc * 32), 256, 0, s>>>(npc, sinv, tc, zc);
    k_cc_prolong_sub<<<nb(c->n_pdof), 256, 0, s>>>(c->n_pdof, c->res[0], agg, ncx, zc, z);
    UWG_CUDA(c, cudaGetLastError());
    return UWG_OK;
}
