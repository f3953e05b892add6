#include "uwg_scan.cuh"

__global__ void k_scan_block(int64_t n, const int32_t* in, int32_t* out, int32_t* bsum) {
    __shared__ int32_t ws[32];
    int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    int32_t v = i < n ? in[i] : 0;
    int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    int32_t x = v;
    for (int o = 1; o < 32; o <<= 1) {
        int32_t y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) ws[w] = x;
    __syncthreads();
    if (w == 0) {
        int32_t t = lane < (int)(blockDim.x >> 5) ? ws[lane] : 0;
        for (int o = 1; o < 32; o <<= 1) {
            int32_t y = __shfl_up_sync(0xffffffffu, t, o);
            if (lane >= o) t += y;
        }
        ws[lane] = t;
    }
    __syncthreads();
    int32_t incl = x + (w > 0 ? ws[w - 1] : 0);
    if (i < n) out[i] = incl - v;
    if (threadIdx.x == blockDim.x - 1) bsum[blockIdx.x] = incl;
}

__global__ void k_scan_add(int64_t n, int32_t* out, const int32_t* boff) {
    int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i < n && blockIdx.x > 0) out[i] += boff[blockIdx.x];
}

int uwg_scan_exclusive(uwg_ctx* c, const int32_t* in, int32_t* out, int64_t n) {
    const int T = 1024;
    if (n <= 0) return UWG_OK;
    int64_t nb = (n + T - 1) / T;
    int32_t* bs = nullptr;
    UWG_CUDA(c, cudaMallocAsync((void**)&bs, (size_t)nb * 2 * 4 + 8, c->stream));
    k_scan_block<<<(unsigned)nb, T, 0, c->stream>>>(n, in, out, bs);
    cudaError_t e = cudaGetLastError();
    int rc = UWG_OK;
    if (e != cudaSuccess) rc = uwg_set_error(c, UWG_ERR_CUDA, cudaGetErrorString(e));
    if (!rc && nb > 1) {
        rc = uwg_scan_exclusive(c, bs, bs + nb, nb);
        if (!rc) {
            k_scan_add<<<(unsigned)nb, T, 0, c->stream>>>(n, out, bs + nb);
            e = cudaGetLastError();
            if (e != cudaSuccess) rc = uwg_set_error(c, UWG_ERR_CUDA, cudaGetErrorString(e));
        }
    }
    cudaFreeAsync(bs, c->stream);
    return rc;
}
