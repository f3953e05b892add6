// Kernels of the learned warm start: a small convolutional network trained on
// solves of the Stokes path itself (no counterpart in the reference).
//
// Every convolution is a GEMM on BF16 tensor cores with FP32 accumulation:
// forward C = im2col(x) W^T, data gradient dcol = dZ W followed by col2im,
// weight gradient dW = dZ^T im2col(x).  Activations are NHWC so that the
// GEMM's K dimension (tap, channel) is contiguous.  The forward product (both
// operands K-major) runs on tcgen05.mma with the accumulator in tensor memory;
// a generic mma.sync m16n8k16 GEMM with optional operand transposes serves the
// two gradient products and operands whose rows are not 16-byte aligned (the
// 3-channel input layer).  Both have a fused bias + ReLU epilogue and FP32 /
// BF16 outputs.
#include <cuda_bf16.h>

#include <algorithm>
#include <cmath>
#include <cstdint>

#include "uwg_internal.cuh"

namespace {

constexpr int BM = 64, BN = 64, BK = 32, PAD = 8;

__device__ __forceinline__ uint32_t ld_pair(const __nv_bfloat16* p) { return *reinterpret_cast<const uint32_t*>(p); }

__device__ __forceinline__ void mma_bf16(float* c, const uint32_t* a, const uint32_t* b) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};\n"
        : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

// C[m][n] (+)= sum_k A(m,k) B(k,n) (+ bias[n]) (ReLU)
//   A(m,k) = AT ? A[k*lda + m] : A[m*lda + k];  B(k,n) = BT ? B[n*ldb + k] : B[k*ldb + n]
// 128 threads, 64x64 tile, each warp 32x32 (2 x 4 mma tiles).  Loads are bounds
// checked element by element (zero outside), stores are bounds checked.
template <bool AT, bool BT>
__global__ void __launch_bounds__(128) k_gemm_bf16(int M, int N, int K, const __nv_bfloat16* __restrict__ A,
                                                   int64_t lda, const __nv_bfloat16* __restrict__ B, int64_t ldb,
                                                   float* Cf, __nv_bfloat16* Cb, int64_t ldc,
                                                   const float* __restrict__ bias, int relu, int accumulate) {
    __shared__ __align__(16) __nv_bfloat16 As[BM][BK + PAD];
    __shared__ __align__(16) __nv_bfloat16 Bs[BN][BK + PAD];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int wm = warp >> 1, wn = warp & 1, g = lane >> 2, t = lane & 3;
    const int m0 = blockIdx.y * BM, n0 = blockIdx.x * BN;
    float acc[2][4][4];
#pragma unroll
    for (int i = 0; i < 2; i++)
#pragma unroll
        for (int j = 0; j < 4; j++)
#pragma unroll
            for (int r = 0; r < 4; r++) acc[i][j][r] = 0.f;
    const __nv_bfloat16 zero = __float2bfloat16(0.f);
    for (int k0 = 0; k0 < K; k0 += BK) {
        // stage A (BM x BK) and B (BN x BK, k contiguous)
        for (int idx = tid; idx < BM * BK; idx += 128) {
            int mm, kk;
            if (AT) { mm = idx % BM; kk = idx / BM; } else { kk = idx % BK; mm = idx / BK; }
            const int gm = m0 + mm, gk = k0 + kk;
            __nv_bfloat16 v = zero;
            if (gm < M && gk < K) v = AT ? A[(int64_t)gk * lda + gm] : A[(int64_t)gm * lda + gk];
            As[mm][kk] = v;
        }
        for (int idx = tid; idx < BN * BK; idx += 128) {
            int nn, kk;
            if (BT) { kk = idx % BK; nn = idx / BK; } else { nn = idx % BN; kk = idx / BN; }
            const int gn = n0 + nn, gk = k0 + kk;
            __nv_bfloat16 v = zero;
            if (gn < N && gk < K) v = BT ? B[(int64_t)gn * ldb + gk] : B[(int64_t)gk * ldb + gn];
            Bs[nn][kk] = v;
        }
        __syncthreads();
#pragma unroll
        for (int kk = 0; kk < BK; kk += 16) {
            uint32_t af[2][4], bf[4][2];
#pragma unroll
            for (int i = 0; i < 2; i++) {
                const int r = wm * 32 + i * 16 + g;
                af[i][0] = ld_pair(&As[r][kk + 2 * t]);
                af[i][1] = ld_pair(&As[r + 8][kk + 2 * t]);
                af[i][2] = ld_pair(&As[r][kk + 2 * t + 8]);
                af[i][3] = ld_pair(&As[r + 8][kk + 2 * t + 8]);
            }
#pragma unroll
            for (int j = 0; j < 4; j++) {
                const int cn = wn * 32 + j * 8 + g;
                bf[j][0] = ld_pair(&Bs[cn][kk + 2 * t]);
                bf[j][1] = ld_pair(&Bs[cn][kk + 2 * t + 8]);
            }
#pragma unroll
            for (int i = 0; i < 2; i++)
#pragma unroll
                for (int j = 0; j < 4; j++) mma_bf16(acc[i][j], af[i], bf[j]);
        }
        __syncthreads();
    }
#pragma unroll
    for (int i = 0; i < 2; i++)
#pragma unroll
        for (int j = 0; j < 4; j++)
#pragma unroll
            for (int r = 0; r < 4; r++) {
                const int gm = m0 + wm * 32 + i * 16 + g + (r >= 2 ? 8 : 0);
                const int gn = n0 + wn * 32 + j * 8 + 2 * t + (r & 1);
                if (gm >= M || gn >= N) continue;
                float v = acc[i][j][r];
                const int64_t o = (int64_t)gm * ldc + gn;
                if (accumulate && Cf) v += Cf[o];
                if (bias) v += bias[gn];
                if (relu) v = fmaxf(v, 0.f);
                if (Cf) Cf[o] = v;
                if (Cb) Cb[o] = __float2bfloat16(v);
            }
}

// ---------------------------------------------------------------------------
// The same product on the 5th-generation tensor cores (tcgen05) for K-major A
// and K-major B (A(m,k) = A[m*lda + k], B(k,n) = B[n*ldb + k]): the
// convolution forward product im2col(x) W^T.
//
// One CTA of 128 threads computes a 128 x BN tile of C.  K advances in chunks
// of 64; each chunk of A (128 x 64) and B (BN x 64) is staged by cp.async into
// shared memory in the no-swizzle K-major core-matrix layout (8 rows x 16 bytes
// per core matrix, 128 contiguous bytes; core matrix (row group g, k group j)
// at (g * 8 + j) * 128 bytes, so the descriptor's leading (K) byte offset is
// 128 and its stride (row-group) byte offset 1024).  Thread 0 issues four
// tcgen05.mma (M 128, N BN, K 16) per chunk into an FP32 accumulator in tensor
// memory and commits them to the chunk buffer's mbarrier; two buffers let the
// next chunk's copies overlap the tensor-core work.  The epilogue reads the
// accumulator back with tcgen05.ld (warp w owns lanes 32w..32w+31 = rows) and
// applies accumulate / bias / ReLU as the mma.sync kernel does.
//
// Every mbarrier wait is bounded (about two seconds of SM clock); a wait that
// gives up sets bit 0 of the status word, the CTA skips the remaining MMAs and
// the epilogue, waits (bounded) for what it has issued, frees its tensor
// memory and returns.
// ---------------------------------------------------------------------------
constexpr int TC_BM = 128, TC_BK = 64;
constexpr long long TC_WAIT_CYCLES = 4000000000LL;

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void tc_cp16(uint32_t dst, const void* src, bool valid) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(dst), "l"(src), "r"(valid ? 16 : 0)
                 : "memory");
}

__device__ __forceinline__ bool tc_wait(uint32_t mbar, uint32_t parity) {
    const long long t0 = clock64();
    while (true) {
        uint32_t done;
        asm volatile(
            "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
            : "=r"(done)
            : "r"(mbar), "r"(parity)
            : "memory");
        if (done) return true;
        if (clock64() - t0 > TC_WAIT_CYCLES) return false;
    }
}

// shared-memory matrix descriptor: start, leading (K) and stride (row group)
// byte offsets in 16-byte units, fixed field 0b001 at bits 46-48, no swizzle
__device__ __forceinline__ uint64_t tc_desc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
    return (uint64_t)((addr >> 4) & 0x3FFF) | ((uint64_t)((lbo >> 4) & 0x3FFF) << 16) |
           ((uint64_t)((sbo >> 4) & 0x3FFF) << 32) | ((uint64_t)1 << 46);
}

template <int BN>
__global__ void __launch_bounds__(128) k_gemm_bf16_tc(int M, int N, int K, const __nv_bfloat16* __restrict__ A,
                                                      int64_t lda, const __nv_bfloat16* __restrict__ B, int64_t ldb,
                                                      float* Cf, __nv_bfloat16* Cb, int64_t ldc,
                                                      const float* __restrict__ bias, int relu, int accumulate,
                                                      int32_t* status) {
    static_assert(BN % 16 == 0 && BN >= 32 && BN <= 256 && (BN & (BN - 1)) == 0, "tensor memory columns");
    constexpr int A_BYTES = TC_BM * TC_BK * 2, B_BYTES = BN * TC_BK * 2, BUF = A_BYTES + B_BYTES;
    // D F32 (bits 4-5 = 1), A BF16 (bits 7-9 = 1), B BF16 (bits 10-12 = 1), both K-major,
    // N >> 3 at bits 17-22, M >> 4 at bits 24-28
    constexpr uint32_t IDESC = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(BN >> 3) << 17) |
                               ((uint32_t)(TC_BM >> 4) << 24);
    extern __shared__ __align__(128) unsigned char tc_smem[];
    __shared__ __align__(8) uint64_t mbar[2];
    __shared__ uint32_t tmem_slot;
    __shared__ int abort_all;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int m0 = blockIdx.y * TC_BM, n0 = blockIdx.x * BN;
    const uint32_t sbase = smem_u32(tc_smem);
    const uint32_t mb0 = smem_u32(&mbar[0]), mb1 = smem_u32(&mbar[1]);

    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(smem_u32(&tmem_slot)),
                     "r"(BN)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::: "memory");
    }
    if (tid == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(mb0) : "memory");
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(mb1) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
        abort_all = 0;
    }
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
    const uint32_t tmem = tmem_slot;

    const int nk = (K + TC_BK - 1) / TC_BK;
    bool ok = true;
    int committed = 0;  // chunks whose MMAs were issued and committed (uniform over the CTA)
    for (int it = 0; it < nk; it++) {
        const int buf = it & 1;
        const uint32_t mb = buf ? mb1 : mb0;
        // the buffer is free once the MMAs of chunk it - 2 have completed
        if (it >= 2 && !tc_wait(mb, ((it - 2) >> 1) & 1)) ok = false;
        if (__syncthreads_or(!ok)) { ok = false; break; }
        committed = it + 1;
        const int k0 = it * TC_BK;
        const uint32_t sa = sbase + buf * BUF, sb = sa + A_BYTES;
        for (int q = tid; q < TC_BM * 8; q += 128) {
            const int r = q >> 3, j = q & 7, gm = m0 + r, gk = k0 + j * 8;
            const bool v = gm < M && gk < K;
            tc_cp16(sa + ((r >> 3) * 8 + j) * 128 + (r & 7) * 16, v ? (const void*)(A + (int64_t)gm * lda + gk) : A, v);
        }
        for (int q = tid; q < BN * 8; q += 128) {
            const int r = q >> 3, j = q & 7, gn = n0 + r, gk = k0 + j * 8;
            const bool v = gn < N && gk < K;
            tc_cp16(sb + ((r >> 3) * 8 + j) * 128 + (r & 7) * 16, v ? (const void*)(B + (int64_t)gn * ldb + gk) : B, v);
        }
        asm volatile("cp.async.wait_all;\n" ::: "memory");
        asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
        __syncthreads();
        if (tid == 0) {
            asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
#pragma unroll
            for (int s = 0; s < TC_BK / 16; s++) {
                const uint64_t da = tc_desc(sa + s * 256, 128, 1024), db = tc_desc(sb + s * 256, 128, 1024);
                const uint32_t acc = (it > 0 || s > 0) ? 1u : 0u;
                asm volatile(
                    "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
                    " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem),
                    "l"(da), "l"(db), "r"(IDESC), "r"(acc)
                    : "memory");
            }
            asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(mb)
                         : "memory");
        }
    }
    // wait for the last commit on each buffer: every MMA this CTA issued has completed
    bool fin = true;
    if (committed >= 1 && !tc_wait((committed - 1) & 1 ? mb1 : mb0, ((committed - 1) >> 1) & 1)) fin = false;
    if (committed >= 2 && !tc_wait((committed - 2) & 1 ? mb1 : mb0, ((committed - 2) >> 1) & 1)) fin = false;
    if (tid == 0 && (!ok || !fin)) {
        atomicOr(status, 1);
        abort_all = 1;
    }
    __syncthreads();
    if (!abort_all) {
        asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
        const int row = m0 + warp * 32 + lane;
#pragma unroll 1
        for (int c0 = 0; c0 < BN; c0 += 16) {
            uint32_t v[16];
            asm volatile(
                "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, "
                "[%16];\n"
                : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]),
                  "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]),
                  "=r"(v[15])
                : "r"(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c0)
                : "memory");
            asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
            if (row >= M) continue;
#pragma unroll
            for (int j = 0; j < 16; j++) {
                const int gn = n0 + c0 + j;
                if (gn >= N) break;
                float x = __uint_as_float(v[j]);
                const int64_t o = (int64_t)row * ldc + gn;
                if (accumulate && Cf) x += Cf[o];
                if (bias) x += bias[gn];
                if (relu) x = fmaxf(x, 0.f);
                if (Cf) Cf[o] = x;
                if (Cb) Cb[o] = __float2bfloat16(x);
            }
        }
    }
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
    __syncthreads();
    if (warp == 0) {
        asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem), "r"(BN) : "memory");
    }
}

// col[p][tap*C + c] = x[pixel p shifted by tap][c] (zero outside), 3x3 taps, NHWC
__global__ void k_im2col(int nb, int H, int W, int C, const __nv_bfloat16* __restrict__ x, __nv_bfloat16* col) {
    const int64_t total = (int64_t)nb * H * W * 9 * C;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x) {
        const int c = (int)(i % C);
        const int tap = (int)((i / C) % 9);
        const int64_t p = i / (9 * (int64_t)C);
        const int xx = (int)(p % W), yy = (int)((p / W) % H);
        const int64_t b = p / ((int64_t)W * H);
        const int sy = yy + tap / 3 - 1, sx = xx + tap % 3 - 1;
        __nv_bfloat16 v = __float2bfloat16(0.f);
        if (sy >= 0 && sy < H && sx >= 0 && sx < W) v = x[((b * H + sy) * W + sx) * C + c];
        col[i] = v;
    }
}

// out[p][c] = sum_tap col[p - shift(tap)][tap][c]: the transpose of k_im2col
__global__ void k_col2im(int nb, int H, int W, int C, const float* __restrict__ col, float* out) {
    const int64_t total = (int64_t)nb * H * W * C;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x) {
        const int c = (int)(i % C);
        const int64_t p = i / C;
        const int xx = (int)(p % W), yy = (int)((p / W) % H);
        const int64_t b = p / ((int64_t)W * H);
        float s = 0.f;
#pragma unroll
        for (int tap = 0; tap < 9; tap++) {
            const int qy = yy - (tap / 3 - 1), qx = xx - (tap % 3 - 1);
            if (qy < 0 || qy >= H || qx < 0 || qx >= W) continue;
            s += col[(((b * H + qy) * W + qx) * 9 + tap) * (int64_t)C + c];
        }
        out[i] = s;
    }
}

__global__ void k_relu_bwd(int64_t n, const __nv_bfloat16* __restrict__ y, float* g) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        if (!(__bfloat162float(y[i]) > 0.f)) g[i] = 0.f;
}

// db[c] = sum_p g[p][c]
__global__ void k_bias_grad(int64_t P, int C, const float* __restrict__ g, float* db) {
    const int c = blockIdx.x;
    float s = 0.f;
    for (int64_t p = threadIdx.x; p < P; p += blockDim.x) s += g[p * C + c];
    __shared__ float red[256];
    red[threadIdx.x] = s;
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
        if ((int)threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) db[c] = red[0];
}

// 2x2 average pooling (H, W even) and its transpose
__global__ void k_pool2(int nb, int H, int W, int C, const __nv_bfloat16* __restrict__ x, __nv_bfloat16* y) {
    const int Ho = H / 2, Wo = W / 2;
    const int64_t total = (int64_t)nb * Ho * Wo * C;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x) {
        const int c = (int)(i % C);
        const int64_t p = i / C;
        const int xo = (int)(p % Wo), yo = (int)((p / Wo) % Ho);
        const int64_t b = p / ((int64_t)Wo * Ho);
        float s = 0.f;
        for (int dy = 0; dy < 2; dy++)
            for (int dx = 0; dx < 2; dx++) s += __bfloat162float(x[((b * H + 2 * yo + dy) * W + 2 * xo + dx) * C + c]);
        y[i] = __float2bfloat16(0.25f * s);
    }
}
__global__ void k_pool2_bwd(int nb, int H, int W, int C, const float* __restrict__ gy, float* gx) {
    const int64_t total = (int64_t)nb * H * W * C;
    const int Ho = H / 2, Wo = W / 2;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x) {
        const int c = (int)(i % C);
        const int64_t p = i / C;
        const int xx = (int)(p % W), yy = (int)((p / W) % H);
        const int64_t b = p / ((int64_t)W * H);
        gx[i] = 0.25f * gy[((b * Ho + yy / 2) * Wo + xx / 2) * C + c];
    }
}

// nearest 2x upsampling and its transpose
__global__ void k_up2(int nb, int H, int W, int C, const __nv_bfloat16* __restrict__ x, __nv_bfloat16* y) {
    const int64_t total = (int64_t)nb * (2 * H) * (2 * W) * C;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x) {
        const int c = (int)(i % C);
        const int64_t p = i / C;
        const int xx = (int)(p % (2 * W)), yy = (int)((p / (2 * W)) % (2 * H));
        const int64_t b = p / ((int64_t)4 * W * H);
        y[i] = x[((b * H + yy / 2) * W + xx / 2) * C + c];
    }
}
__global__ void k_up2_bwd(int nb, int H, int W, int C, const float* __restrict__ gy, float* gx) {
    // H, W: the coarse (input) size
    const int64_t total = (int64_t)nb * H * W * C;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x) {
        const int c = (int)(i % C);
        const int64_t p = i / C;
        const int xx = (int)(p % W), yy = (int)((p / W) % H);
        const int64_t b = p / ((int64_t)W * H);
        float s = 0.f;
        for (int dy = 0; dy < 2; dy++)
            for (int dx = 0; dx < 2; dx++) s += gy[((b * 2 * H + 2 * yy + dy) * (2 * W) + 2 * xx + dx) * C + c];
        gx[i] = s;
    }
}

__global__ void k_add_bf16(int64_t n, const __nv_bfloat16* a, const __nv_bfloat16* b, __nv_bfloat16* y) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        y[i] = __float2bfloat16(__bfloat162float(a[i]) + __bfloat162float(b[i]));
}

__global__ void k_f32_to_bf16(int64_t n, const float* a, __nv_bfloat16* b) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        b[i] = __float2bfloat16(a[i]);
}

// masked mean-squared error over the first nout of C channels: loss partial
// sums into loss[0] and the gradient 2 (y - t) / count
__global__ void k_mse(int64_t P, int C, int nout, const float* __restrict__ y, const float* __restrict__ t,
                      float* g, float* loss, float inv_count) {
    float s = 0.f;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < P * C; i += (int64_t)gridDim.x * blockDim.x) {
        const int c = (int)(i % C);
        float d = 0.f;
        if (c < nout) d = y[i] - t[(i / C) * nout + c];
        g[i] = 2.f * d * inv_count;
        s += d * d;
    }
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if ((threadIdx.x & 31) == 0) atomicAdd(loss, s * inv_count);
}

// Adam on FP32 master weights, BF16 copy refreshed
__global__ void k_adam(int64_t n, float* w, const float* g, float* m, float* v, __nv_bfloat16* wb, float lr, float b1,
                       float b2, float eps, float c1, float c2) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const float gi = g[i];
        const float mi = b1 * m[i] + (1.f - b1) * gi;
        const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
        m[i] = mi;
        v[i] = vi;
        const float wi = w[i] - lr * (mi / c1) / (sqrtf(vi / c2) + eps);
        w[i] = wi;
        if (wb) wb[i] = __float2bfloat16(wi);
    }
}

unsigned grid_for(int64_t n) { return (unsigned)std::min<int64_t>((n + 255) / 256, 152 * 16); }

}  // namespace

// ---------------------------------------------------------------------------
// C ABI (device pointers; BF16 buffers as uint16_t).  All launches on the
// context's stream.
// ---------------------------------------------------------------------------
extern "C" int uwg_cnn_gemm(uwg_ctx* c, int M, int N, int K, const uint16_t* A, int64_t lda, int a_trans,
                            const uint16_t* B, int64_t ldb, int b_trans, float* Cf, uint16_t* Cb, int64_t ldc,
                            const float* bias, int relu, int accumulate) {
    if (!c || M < 0 || N < 0 || K < 0 || !A || !B || (!Cf && !Cb) || (accumulate && !Cf))
        return uwg_set_error(c, UWG_ERR_ARG, "uwg_cnn_gemm: bad argument");
    if (!M || !N) return UWG_OK;
    if ((M + BM - 1) / BM > 65535) return uwg_set_error(c, UWG_ERR_ARG, "uwg_cnn_gemm: M above 65535 x 64 rows");
    const __nv_bfloat16* a = reinterpret_cast<const __nv_bfloat16*>(A);
    const __nv_bfloat16* b = reinterpret_cast<const __nv_bfloat16*>(B);
    __nv_bfloat16* cb = reinterpret_cast<__nv_bfloat16*>(Cb);
    // tcgen05 path: K-major A and B, 16-byte aligned rows (K, lda, ldb multiples of 8)
    const bool tc = c->cnn_path == 0 && !a_trans && b_trans && K > 0 && K % 8 == 0 && lda % 8 == 0 &&
                    ldb % 8 == 0 && ((uintptr_t)A & 15) == 0 && ((uintptr_t)B & 15) == 0;
    if (tc) {
        if (!c->cnn_flag) {
            void* p = nullptr;
            UWG_CUDA(c, cudaMalloc(&p, 16));
            c->cnn_flag = static_cast<int32_t*>(p);   // freed by uwg_ctx_destroy
            UWG_CUDA(c, cudaMemsetAsync(p, 0, 16, c->stream));
        }
        // shared memory per CTA: two chunk buffers (A 16 KB + B BN x 128 B each).  With BN 128 at most
        // three CTAs fit an SM (384 of 512 tensor-memory columns), with BN 64 at most four (256).
        if (N > 64) {
            constexpr int SM = 2 * (TC_BM * TC_BK * 2 + 128 * TC_BK * 2);
            UWG_CUDA(c, cudaFuncSetAttribute(k_gemm_bf16_tc<128>, cudaFuncAttributeMaxDynamicSharedMemorySize, SM));
            dim3 g((N + 127) / 128, (M + TC_BM - 1) / TC_BM);
            k_gemm_bf16_tc<128><<<g, 128, SM, c->stream>>>(M, N, K, a, lda, b, ldb, Cf, cb, ldc, bias, relu, accumulate,
                                                           c->cnn_flag);
        } else {
            constexpr int SM = 2 * (TC_BM * TC_BK * 2 + 64 * TC_BK * 2);
            UWG_CUDA(c, cudaFuncSetAttribute(k_gemm_bf16_tc<64>, cudaFuncAttributeMaxDynamicSharedMemorySize, SM));
            dim3 g((N + 63) / 64, (M + TC_BM - 1) / TC_BM);
            k_gemm_bf16_tc<64><<<g, 128, SM, c->stream>>>(M, N, K, a, lda, b, ldb, Cf, cb, ldc, bias, relu, accumulate,
                                                          c->cnn_flag);
        }
        UWG_CUDA(c, cudaGetLastError());
        return UWG_OK;
    }
    dim3 grid((N + BN - 1) / BN, (M + BM - 1) / BM);
#define G_(AT, BT) k_gemm_bf16<AT, BT><<<grid, 128, 0, c->stream>>>(M, N, K, a, lda, b, ldb, Cf, cb, ldc, bias, relu, accumulate)
    if (a_trans && b_trans) G_(true, true);
    else if (a_trans) G_(true, false);
    else if (b_trans) G_(false, true);
    else G_(false, false);
#undef G_
    UWG_CUDA(c, cudaGetLastError());
    return UWG_OK;
}

extern "C" int uwg_cnn_set_path(uwg_ctx* c, int path) {
    if (!c || path < 0 || path > 1) return uwg_set_error(c, UWG_ERR_ARG, "uwg_cnn_set_path: path 0 or 1");
    c->cnn_path = path;
    return UWG_OK;
}

extern "C" int uwg_cnn_check(uwg_ctx* c) {
    if (!c) return uwg_set_error(c, UWG_ERR_ARG, "uwg_cnn_check: null context");
    UWG_CUDA(c, cudaStreamSynchronize(c->stream));
    if (!c->cnn_flag) return UWG_OK;
    int32_t f = 0;
    UWG_CUDA(c, cudaMemcpy(&f, c->cnn_flag, 4, cudaMemcpyDeviceToHost));
    if (!f) return UWG_OK;
    UWG_CUDA(c, cudaMemset(c->cnn_flag, 0, 4));
    return uwg_set_error(c, UWG_ERR_CUDA, "uwg_cnn_gemm: a tensor-core GEMM wait timed out (output incomplete)");
}

extern "C" int uwg_cnn_im2col(uwg_ctx* c, int nb, int H, int W, int C, const uint16_t* x, uint16_t* col) {
    if (!c || nb < 1 || H < 1 || W < 1 || C < 1 || !x || !col) return uwg_set_error(c, UWG_ERR_ARG, "uwg_cnn_im2col");
    const int64_t n = (int64_t)nb * H * W * 9 * C;
    k_im2col<<<grid_for(n), 256, 0, c->stream>>>(nb, H, W, C, reinterpret_cast<const __nv_bfloat16*>(x),
                                                 reinterpret_cast<__nv_bfloat16*>(col));
    UWG_CUDA(c, cudaGetLastError());
    return UWG_OK;
}

extern "C" int uwg_cnn_col2im(uwg_ctx* c, int nb, int H, int W, int C, const float* col, float* out) {
    if (!c || nb < 1 || H < 1 || W < 1 || C < 1 || !col || !out) return uwg_set_error(c, UWG_ERR_ARG, "uwg_cnn_col2im");
    const int64_t n = (int64_t)nb * H * W * C;
    k_col2im<<<grid_for(n), 256, 0, c->stream>>>(nb, H, W, C, col, out);
    UWG_CUDA(c, cudaGetLastError());
    return UWG_OK;
}

// op: 0 relu_bwd(y=a16, g=f32), 1 pool2(a16->b16), 2 pool2_bwd(fa->fb), 3 up2(a16->b16),
//     4 up2_bwd(fa->fb), 5 add(a16 + b16 -> c16), 6 f32->bf16(fa->b16)
extern "C" int uwg_cnn_elementwise(uwg_ctx* c, int op, int nb, int H, int W, int C, const uint16_t* a16,
                                   const uint16_t* b16, uint16_t* c16, const float* fa, float* fb) {
    if (!c || op < 0 || op > 6) return uwg_set_error(c, UWG_ERR_ARG, "uwg_cnn_elementwise: bad op");
    const int64_t n = (int64_t)nb * H * W * C;
    auto A = reinterpret_cast<const __nv_bfloat16*>(a16);
    auto B = reinterpret_cast<const __nv_bfloat16*>(b16);
    auto Cc = reinterpret_cast<__nv_bfloat16*>(c16);
    switch (op) {
        case 0: k_relu_bwd<<<grid_for(n), 256, 0, c->stream>>>(n, A, fb); break;
        case 1: k_pool2<<<grid_for(n / 4), 256, 0, c->stream>>>(nb, H, W, C, A, Cc); break;
        case 2: k_pool2_bwd<<<grid_for(n), 256, 0, c->stream>>>(nb, H, W, C, fa, fb); break;
        case 3: k_up2<<<grid_for(4 * n), 256, 0, c->stream>>>(nb, H, W, C, A, Cc); break;
        case 4: k_up2_bwd<<<grid_for(n), 256, 0, c->stream>>>(nb, H, W, C, fa, fb); break;
        case 5: k_add_bf16<<<grid_for(n), 256, 0, c->stream>>>(n, A, B, Cc); break;
        case 6: k_f32_to_bf16<<<grid_for(n), 256, 0, c->stream>>>(n, fa, Cc); break;
    }
    UWG_CUDA(c, cudaGetLastError());
    return UWG_OK;
}

extern "C" int uwg_cnn_bias_grad(uwg_ctx* c, int64_t P, int C, const float* g, float* db) {
    if (!c || P < 0 || C < 1 || !g || !db) return uwg_set_error(c, UWG_ERR_ARG, "uwg_cnn_bias_grad");
    k_bias_grad<<<C, 256, 0, c->stream>>>(P, C, g, db);
    UWG_CUDA(c, cudaGetLastError());
    return UWG_OK;
}

extern "C" int uwg_cnn_mse(uwg_ctx* c, int64_t P, int C, int nout, const float* y, const float* t, float* g,
                           float* loss) {
    if (!c || P < 1 || C < 1 || nout < 1 || nout > C || !y || !t || !g || !loss)
        return uwg_set_error(c, UWG_ERR_ARG, "uwg_cnn_mse");
    UWG_CUDA(c, cudaMemsetAsync(loss, 0, sizeof(float), c->stream));
    k_mse<<<grid_for(P * C), 256, 0, c->stream>>>(P, C, nout, y, t, g, loss, 1.f / (float)(P * nout));
    UWG_CUDA(c, cudaGetLastError());
    return UWG_OK;
}

extern "C" int uwg_cnn_adam(uwg_ctx* c, int64_t n, float* w, const float* g, float* m, float* v, uint16_t* wb, float lr,
                            float b1, float b2, float eps, int step) {
    if (!c || n < 0 || !w || !g || !m || !v || step < 1) return uwg_set_error(c, UWG_ERR_ARG, "uwg_cnn_adam");
    const float c1 = 1.f - powf(b1, (float)step), c2 = 1.f - powf(b2, (float)step);
    k_adam<<<grid_for(n), 256, 0, c->stream>>>(n, w, g, m, v, reinterpret_cast<__nv_bfloat16*>(wb), lr, b1, b2, eps, c1,
                                               c2);
    UWG_CUDA(c, cudaGetLastError());
    return UWG_OK;
}
