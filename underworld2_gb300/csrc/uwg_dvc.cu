// Discrete Voronoi cell (DVC) integration weights, one warp per element.
//
// The reference grows every particle's region on a res^dim grid over the
// element, particle by particle and round by round
// (L/PICellerator/Weights/src/DVCWeights.c:676-770): a particle first claims
// cells of its boundary list (free cells, or cells whose owner is strictly
// farther away, :256-365), then rebuilds its boundary list from the cells it
// just claimed (neighbours in the order S, N, E, W, U, D that it does not own,
// each once, :388-486).  Within one particle's step the claims touch distinct
// cells and are independent, and the boundary rebuild is a de-duplicated
// expansion whose order decides nothing (the next claim step again treats its
// cells independently), so the warp performs each step in parallel with
// ballots, prefix counts and atomic bit flags while keeping the reference's
// sequential particle order: results are identical to the sequential algorithm.
//
// Per warp: owner/done bytes and particle coordinates in shared memory,
// boundary lists (double-buffered per round) in a per-warp global scratch.
// Built with -fmad=false (the distance test must round like the reference).
#include <algorithm>

#include "uwg_internal.cuh"

#define DVC_NMAX 128     // particles per element handled by the kernel
#define DVC_WARPS 4      // warps per block

struct dvc_args {
    int64_t n_el;
    int R;               // grid cells per axis
    const int32_t* off;
    double* ip_xi;       // in: local coords, out: centroids (slot order)
    double* ip_w;
    int16_t* scratch;    // per warp: claimed[RC] + pool0[PCAP] + pool1[PCAP]
    int64_t pcap;
    int32_t* status;     // [0] = first error code, [1] = element
    int nmax;            // particle slots per warp in shared memory (<= DVC_NMAX)
};

// Shared memory of one warp for a grid of RC cells and nmax particle slots:
// coordinates, pool headers, FP32 coordinates, the boundary-list membership
// bits (one per cell) and the owner byte of every cell.
__host__ __device__ inline size_t dvc_warp_bytes(int RC, int nmax) {
    size_t b = (size_t)nmax * 3 * 8 + (size_t)nmax * 4 * 4 + (size_t)nmax * 3 * 4 + (size_t)((RC + 31) / 32) * 4 +
               (size_t)RC;
    return (b + 15) & ~(size_t)15;
}

// Dynamic shared-memory limit set on k_dvc by both entry points: the size of the
// largest launch either can make (res 16 in 3D, DVC_NMAX slots).  One fixed
// value means a call on one thread never lowers the limit under a launch of
// the other entry point on another thread.
inline int dvc_smem_limit() { return (int)(192 + dvc_warp_bytes(16 * 16 * 16, DVC_NMAX) * DVC_WARPS); }

__device__ __forceinline__ void dvc_fail(int32_t* status, int code, int64_t el) {
    if (atomicCAS(&status[0], 0, code) == 0) status[1] = (int32_t)el;
}

// Largest particle count of any element (sizes the kernel's shared memory).
__global__ void k_max_count(int64_t n_el, const int32_t* off, int32_t* out) {
    int m = 0;
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n_el; e += (int64_t)gridDim.x * blockDim.x)
        m = max(m, off[e + 1] - off[e]);
    for (int o = 16; o > 0; o >>= 1) m = max(m, __shfl_xor_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0) atomicMax(out, m);
}

// c / R for 0 <= c < 4096 and 1 <= R <= 16 without an integer division: the
// FP32 product c (1/R) is within 5e-4 of the exact quotient, whose fraction
// is a multiple of 1/R >= 1/16, so adding 1e-3 and truncating gives floor(c / R).
__device__ __forceinline__ int dvc_div(int c, float invR) { return (int)__fadd_rn(__fmul_rn((float)c, invR), 1e-3f); }

template <int DIM>
__global__ void __launch_bounds__(32 * DVC_WARPS) k_dvc(dvc_args a) {
    extern __shared__ unsigned char smem[];
    const int R = a.R;
    const int RC = DIM == 3 ? R * R * R : R * R;
    const int NNB = 2 * DIM;
    int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    // per-block cell centre table (accumulated exactly as _DVCWeights_ConstructGrid)
    double* cen = (double*)smem;                       // [16]
    float* cenf = (float*)(cen + 16);                  // [16] FP32 copies
    const int NM = a.nmax;
    unsigned char* wbase = smem + 192 + dvc_warp_bytes(RC, NM) * wib;
    double* xs = (double*)wbase;                       // [NM][3]
    int32_t* hdr = (int32_t*)(xs + NM * 3);            // [2][NM][2] (offset, length) per pool
    float* xf = (float*)(hdr + NM * 4);                // [NM][3] FP32 copies (distance pre-test)
    uint32_t* done = (uint32_t*)(xf + NM * 3);         // [(RC + 31) / 32] bit c: cell c already listed
    uint8_t* owner = (uint8_t*)(done + (RC + 31) / 32); // [RC]
    if (threadIdx.x == 0) {
        double dx = (1.0 - -1.0) / R;
        double X = -1.0 - dx / 2.0;
        for (int i = 0; i < R; i++) { X = X + dx; cen[i] = X; cenf[i] = (float)X; }
    }
    __syncthreads();
    const double dx = (1.0 - -1.0) / R;
    const double da = DIM == 3 ? dx * dx * dx : dx * dx;
    const float invR = 1.0f / (float)R;
    // cell c -> (i, j, k) grid indices
    auto cell_ijk = [&](int c) {
        const int q = dvc_div(c, invR);
        int3 r;
        r.x = c - q * R;
        if (DIM == 3) {
            r.z = dvc_div(q, invR);
            r.y = q - r.z * R;
        } else {
            r.y = q;
            r.z = 0;
        }
        return r;
    };

    int64_t gw = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    int16_t* claimed = a.scratch + gw * (RC + 2 * a.pcap);
    int16_t* pool[2] = {claimed + RC, claimed + RC + a.pcap};
    unsigned lt = (1u << lane) - 1u;

    for (int64_t el = gw; el < a.n_el; el += nw) {
        int32_t o0 = a.off[el];
        int n = a.off[el + 1] - o0;
        if (n == 0) { if (lane == 0) dvc_fail(a.status, UWG_ERR_EMPTY_CELL, el); continue; }
        if (n > NM) { if (lane == 0) dvc_fail(a.status, UWG_ERR_CELL_FULL, el); continue; }
        for (int k = lane; k < n; k += 32) {
            xs[k * 3 + 0] = a.ip_xi[(int64_t)(o0 + k) * DIM + 0];
            xs[k * 3 + 1] = a.ip_xi[(int64_t)(o0 + k) * DIM + 1];
            xs[k * 3 + 2] = DIM == 3 ? a.ip_xi[(int64_t)(o0 + k) * DIM + DIM - 1] : 0.0;
            xf[k * 3 + 0] = (float)xs[k * 3 + 0];
            xf[k * 3 + 1] = (float)xs[k * 3 + 1];
            xf[k * 3 + 2] = (float)xs[k * 3 + 2];
        }
        for (int c = lane; c < RC; c += 32) owner[c] = 0xFF;
        for (int wd = lane; wd < (RC + 31) / 32; wd += 32) done[wd] = 0u;
        __syncwarp();

        int cur = 0;
        int64_t bump = 0;
        bool overflow = false;

        // Boundary rebuild for particle i from claimed[0..ncl) into pool[dst].
        auto update = [&](int i, int ncl, int dst) {
            int64_t start = bump;
            int total = ncl * NNB, cnt = 0;
            for (int base = 0; base < total; base += 32) {
                int t = base + lane;
                int c1 = -1;
                bool ok = false;
                bool keep = false;
                if (t < total) {
                    int c0 = claimed[t / NNB], k = t % NNB;
                    const int3 g = cell_ijk(c0);
                    const int ci = g.x, cj = g.y, ck = g.z;
                    // neighbour k in the order S, N, E, W, U, D, without a divergent switch
                    const int coord = k < 2 ? cj : (k < 4 ? ci : ck);
                    const int stride = k < 2 ? R : (k < 4 ? 1 : R * R);
                    const bool up = k == 1 || k == 2 || k == 4;
                    c1 = (up ? coord < R - 1 : coord > 0) ? c0 + (up ? stride : -stride) : -1;
                    ok = c1 >= 0 && owner[c1] != i && ((done[c1 >> 5] >> (c1 & 31)) & 1u) == 0u;
                    // each cell once: the lane whose OR sets the cell's bit lists it.  The
                    // order inside a boundary list is free: a particle's claims touch
                    // distinct cells and its rebuilt list is a set, so no ownership
                    // decision depends on it.
                    if (ok) {
                        const unsigned bit = 1u << (c1 & 31);
                        keep = (atomicOr(&done[c1 >> 5], bit) & bit) == 0u;
                    }
                }
                unsigned kb = __ballot_sync(0xffffffffu, keep);
                if (keep) {
                    int64_t pos = start + cnt + __popc(kb & lt);
                    if (pos < a.pcap) pool[dst][pos] = (int16_t)c1;
                }
                cnt += __popc(kb);
                __syncwarp();
            }
            if (start + cnt > a.pcap) overflow = true;
            for (int k = lane; k < cnt && start + k < a.pcap; k += 32) {
                const int c = pool[dst][start + k];
                atomicAnd(&done[c >> 5], ~(1u << (c & 31)));
            }
            if (lane == 0) {
                hdr[(dst * NM + i) * 2 + 0] = (int32_t)start;
                hdr[(dst * NM + i) * 2 + 1] = cnt;
            }
            bump = start + cnt;
            __syncwarp();
        };

        // seeding (:687-705 / :735-756): the seed cells of all particles are
        // computed in parallel (same expressions), then claimed in order
        bool bad = false;
        for (int i = lane; i < n; i += 32) {
            // a local coordinate outside [-1, 1] (a particle listed in the wrong
            // element, or a non-finite position) would seed outside the grid:
            // reported, never indexed
            const double vx = (xs[i * 3 + 0] - -1.0) / dx, vy = (xs[i * 3 + 1] - -1.0) / dx;
            const double vz = DIM == 3 ? (xs[i * 3 + 2] - -1.0) / dx : 0.0;
            if (!(vx >= 0.0 && vx < R + 1.0 && vy >= 0.0 && vy < R + 1.0 && vz >= 0.0 && vz < R + 1.0)) {
                bad = true;
                continue;
            }
            int k = (int)vx;
            int j = (int)vy;
            int l = DIM == 3 ? (int)vz : 0;
            if (k == R) k--;
            if (j == R) j--;
            if (DIM == 3 && l == R) l--;
            hdr[(NM + i) * 2] = k + j * R + l * R * R;   // pool-1 headers stay unused until the first growth round
        }
        if (__any_sync(0xffffffffu, bad)) {
            if (lane == 0) dvc_fail(a.status, UWG_ERR_STATE, el);
            continue;
        }
        __syncwarp();
        for (int i = 0; i < n; i++) {
            int c = hdr[(NM + i) * 2];
            if (lane == 0) { owner[c] = (uint8_t)i; claimed[0] = (int16_t)c; }
            __syncwarp();
            update(i, 1, 0);
        }

        // growth rounds (:707-720 / :758-769)
        int rounds = 0;
        while (true) {
            int nxt = cur ^ 1;
            bump = 0;
            int claimed_total = 0;
            for (int i = 0; i < n; i++) {
                int bo = hdr[(cur * NM + i) * 2 + 0], bl = hdr[(cur * NM + i) * 2 + 1];
                int ncl = 0;
                const double px = xs[i * 3 + 0], py = xs[i * 3 + 1], pz = xs[i * 3 + 2];
                const float fpx = xf[i * 3 + 0], fpy = xf[i * 3 + 1], fpz = xf[i * 3 + 2];
                for (int base = 0; base < bl; base += 32) {
                    int t = base + lane;
                    bool take = false;
                    int c0 = 0;
                    if (t < bl) {
                        c0 = pool[cur][bo + t];
                        int o = owner[c0];
                        if (o == 0xFF) take = true;
                        else if (o != i) {
                            // FP32 pre-test: coordinates lie in [-1, 1], so the FP32
                            // value is within 2e-5 of the exact one; only values near
                            // zero need the FP64 expression, whose sign is the result.
                            float fd;
                            const int3 g = cell_ijk(c0);
                            const int ci = g.x, cj = g.y, ck = g.z;
                            {
                                const float fx0 = cenf[ci], fy0 = cenf[cj];
                                const float fx1 = xf[o * 3 + 0], fy1 = xf[o * 3 + 1];
                                fd = (fx1 + fpx - fx0 - fx0) * (fx1 - fpx) + (fy1 + fpy - fy0 - fy0) * (fy1 - fpy);
                                if (DIM == 3) {
                                    const float fz0 = cenf[ck], fz1 = xf[o * 3 + 2];
                                    fd += (fz1 + fpz - fz0 - fz0) * (fz1 - fpz);
                                }
                            }
                            if (fd > 1e-4f) take = true;
                            else if (fd < -1e-4f) take = false;
                            else {
                            double x0 = cen[ci], y0 = cen[cj];
                            double x1 = xs[o * 3 + 0], y1 = xs[o * 3 + 1];
                            double dist;
                            if (DIM == 2) {
                                dist = (x1 + px - x0 - x0) * (x1 - px) + (y1 + py - y0 - y0) * (y1 - py);
                            } else {
                                double z0 = cen[ck], z1 = xs[o * 3 + 2];
                                dist = (x1 + px - x0 - x0) * (x1 - px) + (y1 + py - y0 - y0) * (y1 - py) +
                                       (z1 + pz - z0 - z0) * (z1 - pz);
                            }
                            take = dist > 0.0;
                            }
                        }
                    }
                    unsigned tb = __ballot_sync(0xffffffffu, take);
                    __syncwarp();
                    if (take) {
                        claimed[ncl + __popc(tb & lt)] = (int16_t)c0;
                        owner[c0] = (uint8_t)i;
                    }
                    ncl += __popc(tb);
                    __syncwarp();
                }
                claimed_total += ncl;
                update(i, ncl, nxt);
            }
            cur = nxt;
            rounds++;
            if (rounds > 4 * RC) overflow = true;   // never reached: each claim strictly improves ownership
            if (claimed_total == 0 || overflow) break;
        }
        if (overflow) {
            if (lane == 0) dvc_fail(a.status, UWG_ERR_CELL_FULL, el);
            continue;
        }

        // centroids and weights (:198-254), summed in cell order per particle:
        // a stable counting sort of the cells by owner (into `claimed`, free
        // now) gives every particle its cells in cell order, so each lane sums
        // its own particle's centres in exactly the reference's order.
        int32_t* cnt = hdr;            // [NM]
        int32_t* pos = hdr + NM;       // [NM]
        for (int i = lane; i < n; i += 32) cnt[i] = 0;
        __syncwarp();
        for (int c = lane; c < RC; c += 32) {
            int o = owner[c];
            if (o < n) atomicAdd(&cnt[o], 1);
        }
        __syncwarp();
        if (lane == 0) {
            int run = 0;
            for (int i = 0; i < n; i++) { pos[i] = run; run += cnt[i]; }
        }
        __syncwarp();
        for (int cb = 0; cb < RC; cb += 32) {
            int c = cb + lane;
            int o = c < RC ? owner[c] : 0xFF;
            bool valid = o < n;
            unsigned peers = __match_any_sync(0xffffffffu, valid ? o : 0x100 + lane);
            int p0 = valid ? pos[o] : 0;
            __syncwarp();
            if (valid) {
                claimed[p0 + __popc(peers & lt)] = (int16_t)c;
                if (__ffs(peers) - 1 == lane) pos[o] = p0 + __popc(peers);
            }
            __syncwarp();
        }
        for (int g0 = 0; g0 < n; g0 += 32) {
            int i = g0 + lane;
            if (i < n) {
                const int m = cnt[i], end = pos[i];
                double sx = 0.0, sy = 0.0, sz = 0.0;
                for (int k = end - m; k < end; k++) {
                    const int3 g = cell_ijk(claimed[k]);
                    sx += cen[g.x];
                    sy += cen[g.y];
                    if (DIM == 3) sz += cen[g.z];
                }
                int64_t s = o0 + i;
                a.ip_w[s] = m * da;
                if (m != 0) { sx /= m; sy /= m; sz /= m; }
                a.ip_xi[s * DIM + 0] = sx;
                a.ip_xi[s * DIM + 1] = sy;
                if (DIM == 3) a.ip_xi[s * DIM + DIM - 1] = sz;
            }
        }
        __syncwarp();
    }
}

extern "C" int uwg_dvc_weights(uwg_ctx* c, int res, const int32_t* cell_offsets, double* ip_xi,
                               double* ip_w) {
    if (!c || !cell_offsets || !ip_xi || !ip_w || res < 1 || res > 16)
        return uwg_set_error(c, UWG_ERR_ARG, "uwg_dvc_weights: bad argument (res must be 1..16)");
    int dim = c->dim;
    int RC = dim == 3 ? res * res * res : res * res;
    // size the per-warp particle slots by the fullest element (more warps per SM)
    int32_t* mx = (int32_t*)c->red;
    UWG_CUDA(c, cudaMemsetAsync(mx, 0, 4, c->stream));
    k_max_count<<<(unsigned)std::min<int64_t>((c->n_el + 255) / 256, 4096), 256, 0, c->stream>>>(c->n_el, cell_offsets, mx);
    int32_t nfull = 0;
    UWG_CUDA(c, cudaMemcpyAsync(&nfull, mx, 4, cudaMemcpyDeviceToHost, c->stream));
    UWG_CUDA(c, cudaStreamSynchronize(c->stream));
    const int nmax = std::min(DVC_NMAX, std::max(8, (nfull + 7) & ~7));
    size_t shm = 192 + dvc_warp_bytes(RC, nmax) * DVC_WARPS;
    int dev = 0, nsm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    void (*kern)(dvc_args) = dim == 3 ? k_dvc<3> : k_dvc<2>;
    UWG_CUDA(c, cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, dvc_smem_limit()));
    int per_sm = 0;
    UWG_CUDA(c, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, 32 * DVC_WARPS, shm));
    if (per_sm < 1) per_sm = 1;
    int64_t blocks = std::min<int64_t>((int64_t)nsm * per_sm, (c->n_el + DVC_WARPS - 1) / DVC_WARPS);
    if (blocks < 1) blocks = 1;
    int64_t warps = blocks * DVC_WARPS;
    dvc_args a;
    a.n_el = c->n_el;
    a.R = res;
    a.off = cell_offsets;
    a.ip_xi = ip_xi;
    a.ip_w = ip_w;
    a.pcap = (int64_t)RC * 8;
    a.nmax = nmax;
    void* scratch = nullptr;
    size_t sbytes = (size_t)warps * (RC + 2 * a.pcap) * 2 + 64;
    UWG_CUDA(c, cudaMallocAsync(&scratch, sbytes, c->stream));
    a.scratch = (int16_t*)scratch;
    a.status = (int32_t*)c->red;
    UWG_CUDA(c, cudaMemsetAsync(a.status, 0, 8, c->stream));
    kern<<<(unsigned)blocks, 32 * DVC_WARPS, shm, c->stream>>>(a);
    cudaError_t e = cudaGetLastError();
    int32_t st[2] = {0, 0};
    if (e == cudaSuccess) e = cudaMemcpyAsync(st, a.status, 8, cudaMemcpyDeviceToHost, c->stream);
    cudaFreeAsync(scratch, c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) return uwg_set_error(c, UWG_ERR_CUDA, cudaGetErrorString(e));
    if (st[0] == UWG_ERR_EMPTY_CELL)
        return uwg_set_error(c, UWG_ERR_EMPTY_CELL, "element " + std::to_string(st[1]) +
                             " holds no particle: add more particles per cell");
    if (st[0] == UWG_ERR_CELL_FULL)
        return uwg_set_error(c, UWG_ERR_CELL_FULL, "element " + std::to_string(st[1]) +
                             " exceeds the DVC kernel limits (128 particles per element)");
    if (st[0] == UWG_ERR_STATE)
        return uwg_set_error(c, UWG_ERR_STATE, "element " + std::to_string(st[1]) +
                             " lists a particle whose local coordinates lie outside [-1, 1]");
    return UWG_OK;
}

// ---------------------------------------------------------------------------
// Allocation-free variant of the DVC weights.
//
// Some callers cannot allocate device memory at the point where they need
// the weights: host frameworks that reserve the GPU's memory in their own pool
// when they start and forbid (or cannot satisfy) any later cudaMalloc, and
// plugin hosts that give a plugin device buffers but no allocator.  They cannot
// create a uwg context either, because creating one allocates.  This entry
// point needs neither: the per-warp boundary lists live in the fixed device
// array below, which every GPU that loads libuwg holds until the process exits.
// ---------------------------------------------------------------------------
#include <mutex>

#define UWG_NOALLOC_SCRATCH_BYTES (32u << 20)   // 32 MiB of boundary-list scratch
#define UWG_NOALLOC_MAX_DEVICES 64

static __device__ __align__(256) unsigned char uwg_noalloc_scratch[UWG_NOALLOC_SCRATCH_BYTES + 256];

static std::mutex uwg_noalloc_mutex;
static void* uwg_noalloc_ptr[UWG_NOALLOC_MAX_DEVICES];

extern "C" int uwg_dvc_weights_noalloc(int dim, int res, int64_t n_el, const int32_t* cell_offsets,
                                       double* ip_xi, double* ip_w, void* cuda_stream) {
    if ((dim != 2 && dim != 3) || res < 1 || res > 16 || n_el < 0 || (n_el && (!cell_offsets || !ip_xi || !ip_w)))
        return UWG_ERR_ARG;
    if (n_el == 0) return UWG_OK;
    cudaStream_t stream = (cudaStream_t)cuda_stream;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= UWG_NOALLOC_MAX_DEVICES) return UWG_ERR_CUDA;
    unsigned char* base = nullptr;
    {
        // once per device, with that device current: the device address of the array.
        // The cached address belongs to the device's primary context; it does not
        // survive cudaDeviceReset (the caller must not reset a device between calls).
        std::lock_guard<std::mutex> lock(uwg_noalloc_mutex);
        if (!uwg_noalloc_ptr[dev]) {
            void* p = nullptr;
            if (cudaGetSymbolAddress(&p, uwg_noalloc_scratch) != cudaSuccess || !p) return UWG_ERR_CUDA;
            uwg_noalloc_ptr[dev] = p;
        }
        base = (unsigned char*)uwg_noalloc_ptr[dev];
    }
    int RC = dim == 3 ? res * res * res : res * res;
    size_t shm = 192 + dvc_warp_bytes(RC, DVC_NMAX) * DVC_WARPS;
    dvc_args a;
    a.nmax = DVC_NMAX;
    a.n_el = n_el;
    a.R = res;
    a.off = cell_offsets;
    a.ip_xi = ip_xi;
    a.ip_w = ip_w;
    a.pcap = (int64_t)RC * 8;
    size_t warp_bytes = (size_t)(RC + 2 * a.pcap) * 2;
    int64_t max_warps = (int64_t)(UWG_NOALLOC_SCRATCH_BYTES / warp_bytes);
    int64_t max_blocks = max_warps / DVC_WARPS;
    if (max_blocks < 1) return UWG_ERR_ARG;   // grid too fine for the fixed scratch
    void (*kern)(dvc_args) = dim == 3 ? k_dvc<3> : k_dvc<2>;
    if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, dvc_smem_limit()) != cudaSuccess)
        return UWG_ERR_CUDA;
    int nsm = 0, per_sm = 0;
    if (cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return UWG_ERR_CUDA;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, 32 * DVC_WARPS, shm) != cudaSuccess)
        return UWG_ERR_CUDA;
    int64_t blocks = std::min<int64_t>((int64_t)nsm * std::max(per_sm, 1), (n_el + DVC_WARPS - 1) / DVC_WARPS);
    blocks = std::max<int64_t>(1, std::min(blocks, max_blocks));
    // status word first (must start at zero every call), then the boundary lists
    a.status = (int32_t*)base;
    a.scratch = (int16_t*)(base + 256);
    if (cudaMemsetAsync(a.status, 0, 8, stream) != cudaSuccess) return UWG_ERR_CUDA;
    kern<<<(unsigned)blocks, 32 * DVC_WARPS, shm, stream>>>(a);
    if (cudaGetLastError() != cudaSuccess) return UWG_ERR_CUDA;
    int32_t st[2] = {0, 0};
    if (cudaMemcpyAsync(st, a.status, 8, cudaMemcpyDeviceToHost, stream) != cudaSuccess) return UWG_ERR_CUDA;
    if (cudaStreamSynchronize(stream) != cudaSuccess) return UWG_ERR_CUDA;
    return st[0];   // 0, UWG_ERR_EMPTY_CELL, UWG_ERR_CELL_FULL or UWG_ERR_STATE
}
