// Particle kernels: seeded layout, element search, owner update with the
// reference's cell-table edits, coincident mapping (Newton local coordinates),
// RK2 advection, interpolation and the advection time step.
//
// Built with -fmad=false: every FP64 expression rounds each multiply and add
// in the order written, matching the reference's CPU arithmetic bit for bit.
//
//   L/ = src/underworld/libUnderworld/
#include <algorithm>
#include <cmath>

#include "uwg_geom.cuh"
#include "uwg_scan.cuh"

static uwg_geom make_geom(const uwg_ctx* c) {
    uwg_geom g;
    g.dim = c->dim;
    g.order = c->order;
    for (int d = 0; d < 3; d++) {
        g.res[d] = c->res[d];
        g.nx[d] = d < c->dim ? c->res[d] * c->order + 1 : 1;
        g.minc[d] = c->minc[d];
        g.maxc[d] = c->maxc[d];
        g.ax[d] = c->ax[d];
    }
    return g;
}

// ---------------------------------------------------------------------------
// Park-Miller stream (L/StgDomain/Swarm/src/Random.c:23-53).  Schrage's method
// computes (16807 * s) mod (2^31 - 1) exactly; so does a 64-bit product
// reduced modulo the Mersenne prime, which also gives the jump-ahead
// multiplier 16807^k mod m for each cell's first draw.
// ---------------------------------------------------------------------------
__host__ __device__ __forceinline__ uint64_t pm_mod(uint64_t x) {
    const uint64_t M = 2147483647ull;
    x = (x & M) + (x >> 31);
    x = (x & M) + (x >> 31);
    return x >= M ? x - M : x;
}

__host__ __device__ __forceinline__ uint64_t pm_pow(uint64_t a, uint64_t k) {
    uint64_t r = 1;
    while (k) {
        if (k & 1) r = pm_mod(r * a);
        a = pm_mod(a * a);
        k >>= 1;
    }
    return r;
}

template <int DIM, int ORDER>
__global__ void k_layout_random(uwg_geom g, int64_t n_el, int ppc, uint64_t s0, double* x,
                                int32_t* owner, int32_t* cell_offsets, int32_t* cell_list) {
    constexpr int NEN = Shape<DIM, ORDER>::NEN;
    int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (e > n_el) return;
    cell_offsets[e] = (int32_t)(e * ppc);
    if (e == n_el) return;
    uint64_t s = pm_mod(s0 * pm_pow(16807ull, (uint64_t)e * ppc * DIM));
    int eidx[3];
    el_index(g, e, eidx);
    for (int p = 0; p < ppc; p++) {
        double xi[3], N[NEN];
#pragma unroll
        for (int d = 0; d < DIM; d++) {
            s = pm_mod(s * 16807ull);
            // Swarm_Random_Random_WithMinMax(-1, 1): (max - min) * r / RandMax + min
            xi[d] = (1.0 - -1.0) * (double)s / (double)2147483647 + -1.0;
        }
        Shape<DIM, ORDER>::N(xi, N);
        // FeMesh_CoordLocalToGlobal (L/StgFEM/Discretisation/src/FeMesh.c:333-360)
        double acc[3] = {0.0, 0.0, 0.0};
#pragma unroll
        for (int n = 0; n < NEN; n++)
#pragma unroll
            for (int d = 0; d < DIM; d++) acc[d] += N[n] * node_coord<DIM, ORDER>(g, eidx, n, d);
        int64_t pi = e * ppc + p;
#pragma unroll
        for (int d = 0; d < DIM; d++) x[pi * DIM + d] = acc[d];
        owner[pi] = (int32_t)e;
        cell_list[pi] = (int32_t)pi;
    }
}

template <int DIM>
__global__ void k_locate(uwg_geom g, int64_t n_el, int64_t np, const double* x, int32_t* owner) {
    int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (p >= np) return;
    double pt[3];
#pragma unroll
    for (int d = 0; d < DIM; d++) pt[d] = x[p * DIM + d];
    owner[p] = (int32_t)cell_of<DIM>(g, pt, n_el);
}

// ---------------------------------------------------------------------------
// Owner update (L/StgDomain/Swarm/src/SwarmClass.c:947-1015).
// Sequential semantics: for p = 0..np-1, if the cell changed, remove p from
// its old table by moving the last entry into its slot, then append p to the
// new table.  Tables of different cells never interact, so each cell replays
// its own events (removals and additions, in particle order) on one thread.
// ---------------------------------------------------------------------------
// X: the storage type of the particle coordinates (double, or float with the
// arithmetic still in double).
template <int DIM, typename X>
__global__ void k_owner_events(uwg_geom g, int64_t n_el, int64_t np, const X* x,
                               const int32_t* owner, int32_t* newowner, int32_t* n_events,
                               int32_t* n_add, int32_t* n_rem, unsigned long long* n_lost) {
    int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (p >= np) return;
    double pt[3];
#pragma unroll
    for (int d = 0; d < DIM; d++) pt[d] = (double)x[p * DIM + d];
    int32_t nc = (int32_t)cell_of<DIM>(g, pt, n_el);
    int32_t oc = owner[p];
    newowner[p] = nc;
    if (nc == oc) return;
    if (oc < n_el) {
        atomicAdd(&n_events[oc], 1);
        atomicAdd(&n_rem[oc], 1);
    }
    if (nc < n_el) {
        atomicAdd(&n_events[nc], 1);
        atomicAdd(&n_add[nc], 1);
    } else {
        atomicAdd(n_lost, 1ull);
    }
}

// event code: particle index * 2 + (1 = add, 0 = remove)
__global__ void k_owner_scatter(int64_t n_el, int64_t np, const int32_t* owner, const int32_t* newowner,
                                const int32_t* ev_off, int32_t* ev_fill, int64_t* events) {
    int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (p >= np) return;
    int32_t nc = newowner[p], oc = owner[p];
    if (nc == oc) return;
    if (oc < n_el) {
        int k = atomicAdd(&ev_fill[oc], 1);
        events[ev_off[oc] + k] = p * 2 + 0;
    }
    if (nc < n_el) {
        int k = atomicAdd(&ev_fill[nc], 1);
        events[ev_off[nc] + k] = p * 2 + 1;
    }
}

// new count and temporary capacity per cell
__global__ void k_owner_counts(int64_t n_el, const int32_t* old_off, const int32_t* n_add,
                               const int32_t* n_rem, int32_t* new_cnt, int32_t* tmp_cap) {
    int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (c >= n_el) return;
    int32_t cnt = old_off[c + 1] - old_off[c];
    new_cnt[c] = cnt - n_rem[c] + n_add[c];
    tmp_cap[c] = cnt + n_add[c];
}

__global__ void k_owner_replay(int64_t n_el, const int32_t* old_off, const int32_t* old_list,
                               const int32_t* ev_off, int64_t* events, const int32_t* tmp_off,
                               int32_t* tmp, const int32_t* new_off, int32_t* new_list, int32_t* err) {
    int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (c >= n_el) return;
    int32_t o0 = old_off[c], cnt = old_off[c + 1] - o0;
    int32_t* t = tmp + tmp_off[c];
    for (int k = 0; k < cnt; k++) t[k] = old_list[o0 + k];
    int32_t e0 = ev_off[c], ne = ev_off[c + 1] - e0;
    int64_t* ev = events + e0;
    // insertion sort of this cell's events by particle index
    for (int i = 1; i < ne; i++) {
        int64_t v = ev[i];
        int j = i - 1;
        while (j >= 0 && ev[j] > v) { ev[j + 1] = ev[j]; j--; }
        ev[j + 1] = v;
    }
    for (int i = 0; i < ne; i++) {
        int32_t p = (int32_t)(ev[i] >> 1);
        if (ev[i] & 1) {
            t[cnt++] = p;                       // Swarm_AddParticleToCell: append
        } else {
            int k = 0;                          // Swarm_GetParticleIndexWithinCell
            while (k < cnt && t[k] != p) k++;
            if (k == cnt) { atomicExch(err, 1); return; }
            t[k] = t[cnt - 1];                  // Swarm_RemoveParticleFromCell
            cnt--;
        }
    }
    int32_t n0 = new_off[c];
    if (n0 + cnt != new_off[c + 1]) { atomicExch(err, 2); return; }
    for (int k = 0; k < cnt; k++) new_list[n0 + k] = t[k];
}

__global__ void k_copy_i32(int64_t n, const int32_t* a, int32_t* b) {
    int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i < n) b[i] = a[i];
}

// ---------------------------------------------------------------------------
// Coincident mapping: one thread per cell-table slot.
// ---------------------------------------------------------------------------
__device__ __forceinline__ int64_t slot_element(const int32_t* off, int64_t n_el, int64_t s) {
    int64_t lo = 0, hi = n_el;   // largest e with off[e] <= s
    while (hi - lo > 1) {
        int64_t mid = (lo + hi) >> 1;
        if (off[mid] <= s) lo = mid; else hi = mid;
    }
    return lo;
}

template <int DIM, int ORDER>
__global__ void k_pic_map(uwg_geom g, int64_t n_el, const double* x, const int32_t* off,
                          const int32_t* list, double* ip_xi) {
    int64_t nslots = off[n_el];
    int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (s >= nslots) return;
    int64_t e = slot_element(off, n_el, s);
    int32_t p = list[s];
    int eidx[3];
    el_index(g, e, eidx);
    double pt[3], xi[3];
#pragma unroll
    for (int d = 0; d < DIM; d++) pt[d] = x[(int64_t)p * DIM + d];
    global_to_local<DIM, ORDER>(g, eidx, pt, xi);
#pragma unroll
    for (int d = 0; d < DIM; d++) ip_xi[s * DIM + d] = xi[d];
}

// ---------------------------------------------------------------------------
// Velocity evaluation and RK2.
// ---------------------------------------------------------------------------
// _FeVariable_InterpolateValueAt on a regular mesh (L/StgFEM/Discretisation/src/
// FeVariable.c:389-403, 549-599, 1007-1044).
template <int DIM, int ORDER>
__device__ bool eval_velocity(const uwg_geom& g, const double* vel, const double* pt, double* v) {
    constexpr int NEN = Shape<DIM, ORDER>::NEN;
    constexpr int K = ORDER + 1;
    int eidx[3] = {0, 0, 0};
    if (!search_element<DIM>(g, pt, eidx)) return false;
    double xi[3], N[NEN];
    global_to_local<DIM, ORDER>(g, eidx, pt, xi);
    Shape<DIM, ORDER>::N(xi, N);
#pragma unroll
    for (int d = 0; d < DIM; d++) v[d] = 0.0;
#pragma unroll
    for (int n = 0; n < NEN; n++) {
        int64_t ix = eidx[0] * ORDER + n % K;
        int64_t iy = eidx[1] * ORDER + (n / K) % K;
        int64_t iz = DIM == 3 ? eidx[2] * ORDER + n / (K * K) : 0;
        int64_t node = ix + g.nx[0] * (iy + (int64_t)g.nx[1] * iz);
#pragma unroll
        for (int d = 0; d < DIM; d++) v[d] += vel[node * DIM + d] * N[n];
    }
    if (isinf(v[0]) || isinf(v[1]) || (DIM == 3 && isinf(v[DIM - 1]))) return false;
    return true;
}

// TimeIntegrand_SecondOrder (L/StgDomain/Utils/src/TimeIntegrand.c:249-319) with
// _TimeIntegrand_RewindToStartAndApplyFirstOrderUpdate (:441-468).  X is the
// coordinate storage type: with float storage the stored values are widened to
// double, every step of the update is done in double, and the result is
// rounded once when it is stored.
template <int DIM, int ORDER, typename X>
__global__ void k_rk2(uwg_geom g, int64_t np, double dt, const double* vel, X* x,
                      unsigned long long* counts) {
    int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (p >= np) return;
    double x0[3], xm[3], v[3];
#pragma unroll
    for (int d = 0; d < DIM; d++) x0[d] = (double)x[p * DIM + d];
    if (!eval_velocity<DIM, ORDER>(g, vel, x0, v)) {
        atomicAdd(&counts[1], 1ull);
        return;
    }
#pragma unroll
    for (int d = 0; d < DIM; d++) xm[d] = x0[d] + 0.5 * dt * v[d];
    double vm[3];
    if (eval_velocity<DIM, ORDER>(g, vel, xm, vm)) {
#pragma unroll
        for (int d = 0; d < DIM; d++) x[p * DIM + d] = (X)(x0[d] + dt * vm[d]);
    } else {
        atomicAdd(&counts[0], 1ull);
#pragma unroll
        for (int d = 0; d < DIM; d++) x[p * DIM + d] = (X)(x0[d] + dt * v[d]);
    }
}

template <int DIM, int ORDER>
__global__ void k_interpolate(uwg_geom g, int64_t n, const double* pts, const double* vel, double* out) {
    int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    double pt[3], v[3];
#pragma unroll
    for (int d = 0; d < DIM; d++) pt[d] = pts[i * DIM + d];
    bool ok = eval_velocity<DIM, ORDER>(g, vel, pt, v);
#pragma unroll
    for (int d = 0; d < DIM; d++) out[i * DIM + d] = ok ? v[d] : nan("");
}

// max |v| over nodes (FieldVariable_GetMaxGlobalFieldMagnitude,
// L/StgFEM/Discretisation/src/FeVariable.c:409-437,453-468): the maximum of
// correctly rounded values is order independent, so a tree reduction is exact.
template <int DIM>
__global__ void k_max_speed(int64_t n, const double* vel, unsigned long long* out) {
    __shared__ double sm[32];
    double m = 0.0;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x) {
        double s = 0.0;
#pragma unroll
        for (int d = 0; d < DIM; d++) s += vel[i * DIM + d] * vel[i * DIM + d];
        m = fmax(m, sqrt(s));
    }
    for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0) sm[threadIdx.x >> 5] = m;
    __syncthreads();
    if (threadIdx.x < 32) {
        m = threadIdx.x < (blockDim.x >> 5) ? sm[threadIdx.x] : 0.0;
        for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
        // non-negative doubles order like their bit patterns
        if (threadIdx.x == 0) atomicMax(out, (unsigned long long)__double_as_longlong(m));
    }
}

// ---------------------------------------------------------------------------
// Host entry points
// ---------------------------------------------------------------------------
static inline unsigned nblk(int64_t n, int t = 256) { return (unsigned)((n + t - 1) / t); }

#define UWG_DISPATCH(c, CALL)                                                  \
    do {                                                                        \
        if ((c)->dim == 2 && (c)->order == 1) { CALL(2, 1); }                   \
        else if ((c)->dim == 3 && (c)->order == 1) { CALL(3, 1); }              \
        else if ((c)->dim == 2 && (c)->order == 2) { CALL(2, 2); }              \
        else if ((c)->dim == 3 && (c)->order == 2) { CALL(3, 2); }              \
        else return uwg_set_error(c, UWG_ERR_ARG, "element type not supported"); \
    } while (0)

extern "C" int uwg_layout_random(uwg_ctx* c, int ppc, int64_t* rng_state_h, double* x, int32_t* owner,
                                 int32_t* cell_offsets, int32_t* cell_list) {
    if (!c || !rng_state_h || !x || !owner || !cell_offsets || !cell_list || ppc <= 0)
        return uwg_set_error(c, UWG_ERR_ARG, "uwg_layout_random: bad argument");
    int64_t s0 = *rng_state_h;
    if (s0 <= 0 || s0 >= 2147483647) return uwg_set_error(c, UWG_ERR_ARG, "rng state outside (0, 2^31-1)");
    uwg_geom g = make_geom(c);
#define L_(D, O) k_layout_random<D, O><<<nblk(c->n_el + 1), 256, 0, c->stream>>>(g, c->n_el, ppc, (uint64_t)s0, x, owner, cell_offsets, cell_list)
    UWG_DISPATCH(c, L_);
#undef L_
    UWG_CUDA(c, cudaGetLastError());
    *rng_state_h = (int64_t)pm_mod((uint64_t)s0 * pm_pow(16807ull, (uint64_t)c->n_el * ppc * c->dim));
    return UWG_OK;
}

// Material particle of every Gauss integration point, as GeneralSwarm_IntegrationPointMap
// finds it when a swarm variable is evaluated on a Gauss integration swarm
// (L/PICellerator/MaterialPoints/src/GeneralSwarm.cpp:319-431): the point's global
// position by FeMesh_CoordLocalToGlobal, then the first particle of its element's
// list at the least squared distance.  pid = -1 where the element holds no particle.
// One thread per (element, point); t = e * nq + q.
template <int DIM, int ORDER>
__global__ void k_gauss_nearest(uwg_geom g, int64_t n_el, int nq, const double* xi_q, const int32_t* off,
                                const int32_t* lst, const double* x, int32_t* pid) {
    constexpr int NEN = Shape<DIM, ORDER>::NEN;
    int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (t >= n_el * nq) return;
    int64_t e = t / nq;
    int q = (int)(t - e * nq);
    int eidx[3];
    el_index(g, e, eidx);
    double N[NEN];
    Shape<DIM, ORDER>::N(xi_q + q * DIM, N);
    double pt[3] = {0.0, 0.0, 0.0};
#pragma unroll
    for (int n = 0; n < NEN; n++)
#pragma unroll
        for (int d = 0; d < DIM; d++) pt[d] += N[n] * node_coord<DIM, ORDER>(g, eidx, n, d);
    double best = 1.7976931348623157e308;
    int32_t bi = -1;
    for (int32_t k = off[e]; k < off[e + 1]; k++) {
        const int32_t i = lst[k];
        double d2 = 0.0;
#pragma unroll
        for (int d = 0; d < DIM; d++) {
            const double dd = pt[d] - x[(int64_t)i * DIM + d];
            d2 += dd * dd;
        }
        if (d2 < best) {
            best = d2;
            bi = i;
        }
    }
    pid[t] = bi;
}

extern "C" int uwg_gauss_nearest(uwg_ctx* c, int nq, const double* xi_q, const int32_t* cell_offsets,
                                 const int32_t* cell_list, const double* x, int32_t* pid) {
    if (!c || nq < 1 || !xi_q || !cell_offsets || !cell_list || !x || !pid)
        return uwg_set_error(c, UWG_ERR_ARG, "uwg_gauss_nearest: bad argument");
    const int64_t n = c->n_el * (int64_t)nq;
    uwg_geom g = make_geom(c);
    if (c->dim == 2) {
        if (c->order == 1) k_gauss_nearest<2, 1><<<nblk(n), 256, 0, c->stream>>>(g, c->n_el, nq, xi_q, cell_offsets, cell_list, x, pid);
        else k_gauss_nearest<2, 2><<<nblk(n), 256, 0, c->stream>>>(g, c->n_el, nq, xi_q, cell_offsets, cell_list, x, pid);
    } else {
        if (c->order == 1) k_gauss_nearest<3, 1><<<nblk(n), 256, 0, c->stream>>>(g, c->n_el, nq, xi_q, cell_offsets, cell_list, x, pid);
        else k_gauss_nearest<3, 2><<<nblk(n), 256, 0, c->stream>>>(g, c->n_el, nq, xi_q, cell_offsets, cell_list, x, pid);
    }
    UWG_CUDA(c, cudaGetLastError());
    return UWG_OK;
}

extern "C" int uwg_locate(uwg_ctx* c, int64_t np, const double* x, int32_t* owner) {
    if (!c || np < 0 || (np && (!x || !owner))) return uwg_set_error(c, UWG_ERR_ARG, "uwg_locate: bad argument");
    if (!np) return UWG_OK;
    uwg_geom g = make_geom(c);
    if (c->dim == 2) k_locate<2><<<nblk(np), 256, 0, c->stream>>>(g, c->n_el, np, x, owner);
    else k_locate<3><<<nblk(np), 256, 0, c->stream>>>(g, c->n_el, np, x, owner);
    UWG_CUDA(c, cudaGetLastError());
    return UWG_OK;
}

struct uwg_dev_buf {
    void* p = nullptr;
    ~uwg_dev_buf() { if (p) cudaFree(p); }
};

template <typename X>
static int update_owners(uwg_ctx* c, int64_t np, const X* x, int32_t* owner, int32_t* cell_offsets,
                         int32_t* cell_list, int64_t* n_lost_h) {
    if (!c || np < 0 || !cell_offsets || (np && (!x || !owner || !cell_list)))
        return uwg_set_error(c, UWG_ERR_ARG, "uwg_update_owners: bad argument");
    int64_t n_el = c->n_el;
    uwg_geom g = make_geom(c);
    cudaStream_t s = c->stream;
    // scratch: counts (4 x n_el+1 int32), offsets, events, temp tables
    int64_t ne1 = n_el + 1;
    uwg_dev_buf b_i32, b_ev, b_tmp;
    size_t i32_words = (size_t)ne1 * 7 + (size_t)np + 4;
    UWG_CUDA(c, cudaMallocAsync(&b_i32.p, i32_words * 4 + 16, s));
    int32_t* n_events = (int32_t*)b_i32.p;
    int32_t* n_add = n_events + ne1;
    int32_t* n_rem = n_add + ne1;
    int32_t* ev_off = n_rem + ne1;
    int32_t* new_cnt = ev_off + ne1;
    int32_t* tmp_off = new_cnt + ne1;
    int32_t* new_off = tmp_off + ne1;
    int32_t* newowner = new_off + ne1;
    int32_t* err = newowner + np;
    unsigned long long* lost = (unsigned long long*)(((uintptr_t)(err + 2) + 7) & ~(uintptr_t)7);
    UWG_CUDA(c, cudaMemsetAsync(b_i32.p, 0, (size_t)ne1 * 3 * 4, s));
    UWG_CUDA(c, cudaMemsetAsync(err, 0, 24, s));
    if (np) {
        if (c->dim == 2)
            k_owner_events<2, X><<<nblk(np), 256, 0, s>>>(g, n_el, np, x, owner, newowner, n_events, n_add, n_rem, lost);
        else
            k_owner_events<3, X><<<nblk(np), 256, 0, s>>>(g, n_el, np, x, owner, newowner, n_events, n_add, n_rem, lost);
        UWG_CUDA(c, cudaGetLastError());
    }
    // event offsets
    int rc = uwg_scan_exclusive(c, n_events, ev_off, ne1);
    if (rc) return rc;
    int32_t n_ev_total = 0;
    UWG_CUDA(c, cudaMemcpyAsync(&n_ev_total, ev_off + n_el, 4, cudaMemcpyDeviceToHost, s));
    UWG_CUDA(c, cudaStreamSynchronize(s));
    UWG_CUDA(c, cudaMallocAsync(&b_ev.p, (size_t)std::max<int64_t>(n_ev_total, 1) * 8, s));
    UWG_CUDA(c, cudaMemsetAsync(n_events, 0, (size_t)ne1 * 4, s));   // reuse as fill counters
    if (np) {
        k_owner_scatter<<<nblk(np), 256, 0, s>>>(n_el, np, owner, newowner, ev_off, n_events, (int64_t*)b_ev.p);
        UWG_CUDA(c, cudaGetLastError());
    }
    k_owner_counts<<<nblk(n_el), 256, 0, s>>>(n_el, cell_offsets, n_add, n_rem, new_cnt, tmp_off);
    UWG_CUDA(c, cudaGetLastError());
    UWG_CUDA(c, cudaMemsetAsync(new_cnt + n_el, 0, 4, s));
    UWG_CUDA(c, cudaMemsetAsync(tmp_off + n_el, 0, 4, s));
    rc = uwg_scan_exclusive(c, new_cnt, new_off, ne1);
    if (rc) return rc;
    rc = uwg_scan_exclusive(c, tmp_off, tmp_off, ne1);
    if (rc) return rc;
    int32_t tot[2] = {0, 0};
    UWG_CUDA(c, cudaMemcpyAsync(&tot[0], tmp_off + n_el, 4, cudaMemcpyDeviceToHost, s));
    UWG_CUDA(c, cudaMemcpyAsync(&tot[1], new_off + n_el, 4, cudaMemcpyDeviceToHost, s));
    UWG_CUDA(c, cudaStreamSynchronize(s));
    UWG_CUDA(c, cudaMallocAsync(&b_tmp.p, ((size_t)std::max(tot[0], 1) + (size_t)std::max(tot[1], 1)) * 4, s));
    int32_t* tmp = (int32_t*)b_tmp.p;
    int32_t* nlist = tmp + std::max(tot[0], 1);
    k_owner_replay<<<nblk(n_el, 128), 128, 0, s>>>(n_el, cell_offsets, cell_list, ev_off, (int64_t*)b_ev.p,
                                              tmp_off, tmp, new_off, nlist, err);
    UWG_CUDA(c, cudaGetLastError());
    int32_t herr = 0;
    unsigned long long hlost = 0;
    UWG_CUDA(c, cudaMemcpyAsync(&herr, err, 4, cudaMemcpyDeviceToHost, s));
    UWG_CUDA(c, cudaMemcpyAsync(&hlost, lost, 8, cudaMemcpyDeviceToHost, s));
    UWG_CUDA(c, cudaStreamSynchronize(s));
    if (herr) return uwg_set_error(c, UWG_ERR_STATE, "cell tables inconsistent with particle owners");
    if (np) {
        k_copy_i32<<<nblk(np), 256, 0, s>>>(np, newowner, owner);
        UWG_CUDA(c, cudaGetLastError());
    }
    UWG_CUDA(c, cudaMemcpyAsync(cell_offsets, new_off, (size_t)ne1 * 4, cudaMemcpyDeviceToDevice, s));
    if (tot[1] > 0)
        UWG_CUDA(c, cudaMemcpyAsync(cell_list, nlist, (size_t)tot[1] * 4, cudaMemcpyDeviceToDevice, s));
    UWG_CUDA(c, cudaStreamSynchronize(s));
    if (n_lost_h) *n_lost_h = (int64_t)hlost;
    return UWG_OK;
}

extern "C" int uwg_update_owners(uwg_ctx* c, int64_t np, const double* x, int32_t* owner,
                                 int32_t* cell_offsets, int32_t* cell_list, int64_t* n_lost_h) {
    return update_owners<double>(c, np, x, owner, cell_offsets, cell_list, n_lost_h);
}

extern "C" int uwg_update_owners_f32(uwg_ctx* c, int64_t np, const float* x, int32_t* owner,
                                     int32_t* cell_offsets, int32_t* cell_list, int64_t* n_lost_h) {
    return update_owners<float>(c, np, x, owner, cell_offsets, cell_list, n_lost_h);
}

extern "C" int uwg_pic_map(uwg_ctx* c, int64_t np, const double* x, const int32_t* cell_offsets,
                           const int32_t* cell_list, double* ip_xi) {
    if (!c || np < 0 || !cell_offsets || (np && (!x || !cell_list || !ip_xi)))
        return uwg_set_error(c, UWG_ERR_ARG, "uwg_pic_map: bad argument");
    if (!np) return UWG_OK;
    uwg_geom g = make_geom(c);
#define L_(D, O) k_pic_map<D, O><<<nblk(np), 256, 0, c->stream>>>(g, c->n_el, x, cell_offsets, cell_list, ip_xi)
    UWG_DISPATCH(c, L_);
#undef L_
    UWG_CUDA(c, cudaGetLastError());
    return UWG_OK;
}

template <typename X>
static int rk2_advect(uwg_ctx* c, int64_t np, double dt, const double* vel, X* x, int64_t* n_fallback_h,
                      int64_t* n_failed_h) {
    if (!c || np < 0 || !vel || (np && !x)) return uwg_set_error(c, UWG_ERR_ARG, "uwg_rk2_advect: bad argument");
    uwg_geom g = make_geom(c);
    unsigned long long* cnt = (unsigned long long*)c->red;
    UWG_CUDA(c, cudaMemsetAsync(cnt, 0, 16, c->stream));
    if (np) {
#define L_(D, O) k_rk2<D, O, X><<<nblk(np), 256, 0, c->stream>>>(g, np, dt, vel, x, cnt)
        UWG_DISPATCH(c, L_);
#undef L_
        UWG_CUDA(c, cudaGetLastError());
    }
    if (n_fallback_h || n_failed_h) {
        unsigned long long h[2];
        UWG_CUDA(c, cudaMemcpyAsync(h, cnt, 16, cudaMemcpyDeviceToHost, c->stream));
        UWG_CUDA(c, cudaStreamSynchronize(c->stream));
        if (n_fallback_h) *n_fallback_h = (int64_t)h[0];
        if (n_failed_h) *n_failed_h = (int64_t)h[1];
    }
    return UWG_OK;
}

extern "C" int uwg_rk2_advect(uwg_ctx* c, int64_t np, double dt, const double* vel, double* x,
                              int64_t* n_fallback_h, int64_t* n_failed_h) {
    return rk2_advect<double>(c, np, dt, vel, x, n_fallback_h, n_failed_h);
}

extern "C" int uwg_rk2_advect_f32(uwg_ctx* c, int64_t np, double dt, const double* vel, float* x,
                                  int64_t* n_fallback_h, int64_t* n_failed_h) {
    return rk2_advect<float>(c, np, dt, vel, x, n_fallback_h, n_failed_h);
}

extern "C" int uwg_interpolate(uwg_ctx* c, int64_t n, const double* pts, const double* vel, double* out) {
    if (!c || n < 0 || (n && (!pts || !vel || !out))) return uwg_set_error(c, UWG_ERR_ARG, "uwg_interpolate: bad argument");
    if (!n) return UWG_OK;
    uwg_geom g = make_geom(c);
#define L_(D, O) k_interpolate<D, O><<<nblk(n), 256, 0, c->stream>>>(g, n, pts, vel, out)
    UWG_DISPATCH(c, L_);
#undef L_
    UWG_CUDA(c, cudaGetLastError());
    return UWG_OK;
}

// Values (and optionally global gradients) of a nodal field with ncomp
// components at arbitrary points: FeVariable_InterpolateValueAt /
// FeVariable_InterpolateDerivativesAt (L/StgFEM/Discretisation/src/FeVariable.c:549-599,
// 1007-1044) for the function graph's mesh-variable inputs.  Values use
// eval_velocity's arithmetic order (bit-exact with it for ncomp = dim); gradients
// are dN/dxi over the axis-aligned Jacobian, laid out [point][comp][axis].
// Points outside the mesh get NaN.
template <int DIM, int ORDER>
__global__ void k_interp_field(uwg_geom g, int64_t n, const double* __restrict__ pts,
                               const double* __restrict__ field, int ncomp, double* __restrict__ out,
                               double* __restrict__ grad) {
    constexpr int NEN = Shape<DIM, ORDER>::NEN;
    constexpr int K = ORDER + 1;
    int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    double pt[3] = {0.0, 0.0, 0.0};
#pragma unroll
    for (int d = 0; d < DIM; d++) pt[d] = pts[i * DIM + d];
    int eidx[3] = {0, 0, 0};
    if (!search_element<DIM>(g, pt, eidx)) {
        for (int c = 0; c < ncomp; c++) {
            out[i * ncomp + c] = nan("");
            if (grad)
                for (int d = 0; d < DIM; d++) grad[(i * ncomp + c) * DIM + d] = nan("");
        }
        return;
    }
    double xi[3], N[NEN], dN[3][NEN];
    global_to_local<DIM, ORDER>(g, eidx, pt, xi);
    Shape<DIM, ORDER>::N(xi, N);
    int64_t node[NEN];
#pragma unroll
    for (int a = 0; a < NEN; a++) {
        int64_t ix = eidx[0] * ORDER + a % K;
        int64_t iy = eidx[1] * ORDER + (a / K) % K;
        int64_t iz = DIM == 3 ? eidx[2] * ORDER + a / (K * K) : 0;
        node[a] = ix + g.nx[0] * (iy + (int64_t)g.nx[1] * iz);
    }
    double jac[3] = {1.0, 1.0, 1.0};
    if (grad) {
        Shape<DIM, ORDER>::dN(xi, dN);
#pragma unroll
        for (int d = 0; d < DIM; d++) {
            double s = 0.0;
#pragma unroll
            for (int a = 0; a < NEN; a++) s += node_coord<DIM, ORDER>(g, eidx, a, d) * dN[d][a];
            jac[d] = s;
        }
    }
    for (int c = 0; c < ncomp; c++) {
        double v = 0.0;
#pragma unroll
        for (int a = 0; a < NEN; a++) v += field[node[a] * ncomp + c] * N[a];
        out[i * ncomp + c] = v;
        if (grad) {
#pragma unroll
            for (int d = 0; d < DIM; d++) {
                double s = 0.0;
#pragma unroll
                for (int a = 0; a < NEN; a++) s += field[node[a] * ncomp + c] * dN[d][a];
                grad[(i * ncomp + c) * DIM + d] = s / jac[d];
            }
        }
    }
}

extern "C" int uwg_interpolate_field(uwg_ctx* c, int64_t n, const double* pts, const double* field, int ncomp,
                                     double* out, double* grad) {
    if (!c || n < 0 || ncomp < 1 || (n && (!pts || !field || !out)))
        return uwg_set_error(c, UWG_ERR_ARG, "uwg_interpolate_field: bad argument");
    if (!n) return UWG_OK;
    uwg_geom g = make_geom(c);
#define L_(D, O) k_interp_field<D, O><<<nblk(n, 128), 128, 0, c->stream>>>(g, n, pts, field, ncomp, out, grad)
    UWG_DISPATCH(c, L_);
#undef L_
    UWG_CUDA(c, cudaGetLastError());
    return UWG_OK;
}

// ---------------------------------------------------------------------------
// Semi-Lagrangian departure values for SLCN advection-diffusion
// (SemiLagrangianIntegrator_SolveNew, L/StgFEM/Utils/src/SemiLagrangianIntegrator.c:600-653)
// on a Q1 mesh, one thread per node: RK4 back along the velocity (IntegrateRungeKutta,
// :267-302, every stage clamped to the domain by the non-periodic PeriodicUpdate,
// :382-393), then the node value if the launch point lies within 1e-6 minsep of the
// node (:507-532, rtol 0), else the 4^dim Lagrange interpolant (InterpLagrange,
// :357-380) on the static stencil (:534-598) of the element that holds the launch
// point (BicubicInterpolatorNew, :395-505).  Bit-exact with the reference's order.
#define SLCN_INV6 0.166666666667   // the reference's INV6, not 1/6

__device__ __forceinline__ void slcn_clamp(const uwg_geom& g, double* p, int d) {
    if (p[d] < g.minc[d]) { p[d] = g.minc[d]; return; }
    if (p[d] > g.maxc[d]) p[d] = g.maxc[d];
}

__device__ __forceinline__ int slcn_stencil_start(int i, int n) {
    int s = i > 0 ? i - 1 : i;
    s += 3;
    return s >= n ? s - 4 : s - 3;
}

// Lagrange factors of the 4 stencil coordinates at x, in InterpLagrange's order
__device__ __forceinline__ void slcn_factors(double x, const double* c, double* f) {
#pragma unroll
    for (int n = 0; n < 4; n++) {
        double v = 1.0;
#pragma unroll
        for (int o = 0; o < 4; o++) {
            if (o == n) continue;
            v *= (x - c[o]) / (c[n] - c[o]);
        }
        f[n] = v;
    }
}

__device__ __forceinline__ double slcn_dot4(const double* v, const double* f) {
    double r = 0.0;
#pragma unroll
    for (int n = 0; n < 4; n++) r += v[n] * f[n];
    return r;
}

template <int DIM>
__global__ void k_slcn_departure(uwg_geom g, int64_t n_nodes, double dt, const double* __restrict__ vel,
                                 const double* __restrict__ phi, double atol, double* __restrict__ phistar) {
    int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n_nodes) return;
    const int64_t id[3] = {i % g.nx[0], (i / g.nx[0]) % g.nx[1], i / ((int64_t)g.nx[0] * g.nx[1])};
    double x0[3] = {0.0, 0.0, 0.0}, xp[3] = {0.0, 0.0, 0.0}, pos[3] = {0.0, 0.0, 0.0};
    double k[4][3];
#pragma unroll
    for (int s = 0; s < 4; s++) k[s][0] = k[s][1] = k[s][2] = 0.0;
#pragma unroll
    for (int d = 0; d < DIM; d++) x0[d] = g.ax[d][id[d]];
    // the reference ignores the interpolation status: every stage point is inside the domain
    eval_velocity<DIM, 1>(g, vel, x0, k[0]);
#pragma unroll
    for (int d = 0; d < DIM; d++) { xp[d] = x0[d] - 0.5 * dt * k[0][d]; slcn_clamp(g, xp, d); }
    eval_velocity<DIM, 1>(g, vel, xp, k[1]);
#pragma unroll
    for (int d = 0; d < DIM; d++) { xp[d] = x0[d] - 0.5 * dt * k[1][d]; slcn_clamp(g, xp, d); }
    eval_velocity<DIM, 1>(g, vel, xp, k[2]);
#pragma unroll
    for (int d = 0; d < DIM; d++) { xp[d] = x0[d] - dt * k[2][d]; slcn_clamp(g, xp, d); }
    eval_velocity<DIM, 1>(g, vel, xp, k[3]);
#pragma unroll
    for (int d = 0; d < DIM; d++) {
        pos[d] = x0[d] - SLCN_INV6 * dt * (k[0][d] + 2.0 * k[1][d] + 2.0 * k[2][d] + k[3][d]);
        slcn_clamp(g, pos, d);
    }
    double dot = 0.0;
#pragma unroll
    for (int d = DIM - 1; d >= 0; d--) dot = dot + (pos[d] - x0[d]) * (pos[d] - x0[d]);
    int e[3] = {0, 0, 0};
    if (sqrt(dot) < atol || !search_element<DIM>(g, pos, e)) {
        phistar[i] = phi[i];
        return;
    }
    int s[3] = {0, 0, 0};
    double f[3][4];
#pragma unroll
    for (int d = 0; d < DIM; d++) {
        s[d] = slcn_stencil_start(e[d], g.nx[d]);
        double c[4];
#pragma unroll
        for (int a = 0; a < 4; a++) c[a] = g.ax[d][s[d] + a];
        slcn_factors(pos[d], c, f[d]);
    }
    double ptsX[4], ptsY[4], ptsZ[4];
    if (DIM == 2) {
#pragma unroll
        for (int yi = 0; yi < 4; yi++) {
            const double* row = phi + (s[0] + (int64_t)(s[1] + yi) * g.nx[0]);
#pragma unroll
            for (int xi = 0; xi < 4; xi++) ptsX[xi] = row[xi];
            ptsY[yi] = slcn_dot4(ptsX, f[0]);
        }
        phistar[i] = slcn_dot4(ptsY, f[1]);
    } else {
#pragma unroll
        for (int zi = 0; zi < 4; zi++) {
#pragma unroll
            for (int yi = 0; yi < 4; yi++) {
                const double* row = phi + (s[0] + (int64_t)g.nx[0] * ((s[1] + yi) + (int64_t)g.nx[1] * (s[2] + zi)));
#pragma unroll
                for (int xi = 0; xi < 4; xi++) ptsX[xi] = row[xi];
                ptsY[yi] = slcn_dot4(ptsX, f[0]);
            }
            ptsZ[zi] = slcn_dot4(ptsY, f[1]);
        }
        phistar[i] = slcn_dot4(ptsZ, f[2]);
    }
}

extern "C" int uwg_slcn_phistar(uwg_ctx* c, double dt, const double* vel, const double* phi, double* phistar) {
    if (!c || !vel || !phi || !phistar || !(dt == dt))
        return uwg_set_error(c, UWG_ERR_ARG, "uwg_slcn_phistar: bad argument");
    if (c->order != 1) return uwg_set_error(c, UWG_ERR_ARG, "semi-Lagrangian advection is provided on Q1 meshes");
    for (int d = 0; d < c->dim; d++)
        if (c->res[d] < 3)
            return uwg_set_error(c, UWG_ERR_ARG, "semi-Lagrangian stencils need at least 4 nodes per axis");
    uwg_geom g = make_geom(c);
    const double atol = 1e-6 * c->min_sep;
    if (c->dim == 2) k_slcn_departure<2><<<nblk(c->n_nodes, 128), 128, 0, c->stream>>>(g, c->n_nodes, dt, vel, phi, atol, phistar);
    else k_slcn_departure<3><<<nblk(c->n_nodes, 128), 128, 0, c->stream>>>(g, c->n_nodes, dt, vel, phi, atol, phistar);
    UWG_CUDA(c, cudaGetLastError());
    return UWG_OK;
}

extern "C" int uwg_max_dt(uwg_ctx* c, const double* vel, double* dt_h) {
    if (!c || !vel || !dt_h) return uwg_set_error(c, UWG_ERR_ARG, "uwg_max_dt: bad argument");
    unsigned long long* m = (unsigned long long*)c->red;
    UWG_CUDA(c, cudaMemsetAsync(m, 0, 8, c->stream));
    unsigned nb = std::min<unsigned>(nblk(c->n_nodes), 1024u);
    if (c->dim == 2) k_max_speed<2><<<nb, 256, 0, c->stream>>>(c->n_nodes, vel, m);
    else k_max_speed<3><<<nb, 256, 0, c->stream>>>(c->n_nodes, vel, m);
    UWG_CUDA(c, cudaGetLastError());
    unsigned long long hm = 0;
    UWG_CUDA(c, cudaMemcpyAsync(&hm, m, 8, cudaMemcpyDeviceToHost, c->stream));
    UWG_CUDA(c, cudaStreamSynchronize(c->stream));
    double vmax;
    memcpy(&vmax, &hm, 8);
    // SwarmAdvector_MaxDt: localDt = 0.5 * minSeparation / velMax
    *dt_h = 0.5 * c->min_sep / vmax;
    return UWG_OK;
}
