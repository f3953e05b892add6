// Particle deletion and creation with the reference's swarm bookkeeping:
//   * escaped-particle removal (EscapedRoutine_RemoveFromSwarm,
//     L/PICellerator/PopulationControl/src/EscapedRoutine.c:174-284), and
//   * PCDVC population control (_PCDVC_Calculate2D/3D,
//     L/PICellerator/Utils/src/PCDVC.c:313-1084, non-aggressive path): per
//     element, particles whose Voronoi volume exceeds the split threshold are
//     split (a copy at the centroid of their Voronoi cell, appended to the swarm
//     and to the element), those below the delete threshold are deleted.
// The Voronoi volumes and centroids come from uwg_dvc_weights on the GPU.  The
// reference then edits its particle array one operation at a time: a deleted
// particle's slot is refilled by the array's last particle (Swarm_DeleteParticle,
// L/StgDomain/Swarm/src/SwarmClass.c:1032-1085), whose cell-table entry is
// relabelled; a deleted particle leaves its cell by swap-with-last
// (Swarm_RemoveParticleFromCell, :1016-1030); new particles are appended
// (Swarm_AddParticleToCell, :1121-1136).  Elements are processed in order and
// the final particle order depends on every earlier operation, so the plan
// replays those operations on the host (operations, not particles: cost
// proportional to the edits plus one pass over the cell tables) and the GPU
// applies the resulting gather to the particle arrays.  New particle
// coordinates are FeMesh_CoordLocalToGlobal of the centroid, in the
// reference's arithmetic order (this file is built without FMA contraction).
#include <algorithm>
#include <cstring>
#include <unordered_map>
#include <vector>

#include "uwg_geom.cuh"

struct uwg_pop {
    int64_t np_old = 0, np_new = 0;
    std::vector<int32_t> src;        // [np_new] particle whose data each final particle carries
    std::vector<int32_t> owner;      // [np_new]
    std::vector<int32_t> off, lst;   // final cell tables
    std::vector<int32_t> new_index;  // final index of each created particle that survives
    std::vector<int32_t> new_cell;   //   its element
    std::vector<int64_t> new_slot;   //   the ip_xi row holding its local coordinate
};

void uwg_pop_free(uwg_ctx* c) {
    if (c && c->pop) {
        delete (uwg_pop*)c->pop;
        c->pop = nullptr;
    }
}

namespace {

inline unsigned nblk(int64_t n, int t = 256) { return (unsigned)((n + t - 1) / t); }

// Replay of the reference's array and cell-table edits.  ident[i] names the
// particle now at index i: an original index (< N0) or N0 + k for the k-th
// created particle.
struct Replay {
    int64_t N0, count;
    int32_t n_cells;
    std::vector<int64_t> ident;
    const std::vector<int32_t>& owner0;
    const std::vector<int32_t>& off0;
    const std::vector<int32_t>& lst0;
    std::vector<int32_t> new_cell;      // element of created particle k
    std::vector<int64_t> new_slot;      // centroid row of created particle k
    std::vector<int64_t> new_from;      // identity it was split from
    std::unordered_map<int32_t, std::vector<int32_t>> mod;   // edited cell lists

    Replay(int64_t n, int32_t nc, const std::vector<int32_t>& o, const std::vector<int32_t>& f,
           const std::vector<int32_t>& l)
        : N0(n), count(n), n_cells(nc), ident(n), owner0(o), off0(f), lst0(l) {
        for (int64_t i = 0; i < n; i++) ident[i] = i;
    }
    int32_t cell_of(int64_t id) const { return id < N0 ? owner0[id] : new_cell[id - N0]; }
    std::vector<int32_t>& list(int32_t c) {
        auto it = mod.find(c);
        if (it == mod.end())
            it = mod.emplace(c, std::vector<int32_t>(lst0.begin() + off0[c], lst0.begin() + off0[c + 1])).first;
        return it->second;
    }
    bool relabel(int32_t c, int64_t from, int64_t to) {       // Swarm_GetParticleIndexWithinCell + store
        if (c < 0 || c >= n_cells) return false;
        auto& L = list(c);
        for (auto& v : L)
            if (v == from) { v = (int32_t)to; return true; }
        return false;
    }
    // the array part of Swarm_DeleteParticle / EscapedRoutine_RemoveParticles
    bool remove_index(int64_t p) {
        const int64_t last = count - 1;
        if (p != last) {
            const int64_t idl = ident[last];
            if (!relabel(cell_of(idl), last, p)) return false;
            ident[p] = idl;
        }
        count--;
        return true;
    }
    int64_t append(int32_t c, int64_t from_id, int64_t slot) {   // split: Swarm_CreateNewParticle + AddParticleToCell
        const int64_t id = N0 + (int64_t)new_cell.size();
        new_cell.push_back(c);
        new_slot.push_back(slot);
        new_from.push_back(from_id);
        if ((int64_t)ident.size() <= count) ident.resize(count + 1);
        ident[count] = id;
        list(c).push_back((int32_t)count);
        return count++;
    }
    int64_t data_source(int64_t id) const {
        while (id >= N0) id = new_from[id - N0];
        return id;
    }
    void finish(uwg_pop& P) {
        P.np_new = count;
        P.src.resize(count);
        P.owner.resize(count);
        for (int64_t i = 0; i < count; i++) {
            const int64_t id = ident[i];
            P.src[i] = (int32_t)data_source(id);
            P.owner[i] = cell_of(id);
            if (id >= N0) {
                P.new_index.push_back((int32_t)i);
                P.new_cell.push_back(new_cell[id - N0]);
                P.new_slot.push_back(new_slot[id - N0]);
            }
        }
        P.off.assign(n_cells + 1, 0);
        P.lst.clear();
        P.lst.reserve(count);
        for (int32_t c = 0; c < n_cells; c++) {
            auto it = mod.find(c);
            if (it == mod.end()) P.lst.insert(P.lst.end(), lst0.begin() + off0[c], lst0.begin() + off0[c + 1]);
            else P.lst.insert(P.lst.end(), it->second.begin(), it->second.end());
            P.off[c + 1] = (int32_t)P.lst.size();
        }
    }
};

int fetch_tables(uwg_ctx* c, int64_t np, const int32_t* owner, const int32_t* off, const int32_t* lst,
                 std::vector<int32_t>& ho, std::vector<int32_t>& hf, std::vector<int32_t>& hl) {
    ho.resize(np);
    hf.resize(c->n_el + 1);
    if (np) UWG_CUDA(c, cudaMemcpyAsync(ho.data(), owner, sizeof(int32_t) * np, cudaMemcpyDeviceToHost, c->stream));
    UWG_CUDA(c, cudaMemcpyAsync(hf.data(), off, sizeof(int32_t) * (c->n_el + 1), cudaMemcpyDeviceToHost, c->stream));
    UWG_CUDA(c, cudaStreamSynchronize(c->stream));
    if (hf[c->n_el] < 0 || hf[c->n_el] > np) return uwg_set_error(c, UWG_ERR_STATE, "cell tables inconsistent");
    hl.resize(hf[c->n_el]);
    if (!hl.empty())
        UWG_CUDA(c, cudaMemcpyAsync(hl.data(), lst, sizeof(int32_t) * hl.size(), cudaMemcpyDeviceToHost, c->stream));
    UWG_CUDA(c, cudaStreamSynchronize(c->stream));
    return UWG_OK;
}

__global__ void k_pop_gather(int64_t n, int dim, const int32_t* __restrict__ src, const double* __restrict__ x_old,
                             double* __restrict__ x_new) {
    int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int64_t s = src[i];
    for (int d = 0; d < dim; d++) x_new[i * dim + d] = x_old[s * dim + d];
}

// FeMesh_CoordLocalToGlobal (L/StgFEM/Discretisation/src/FeMesh.c:333-360) of the
// split particle's centroid, into its final slot
template <int DIM, int ORDER>
__global__ void k_pop_new_coords(uwg_geom g, int64_t n, const int32_t* __restrict__ idx,
                                 const int32_t* __restrict__ cell, const int64_t* __restrict__ slot,
                                 const double* __restrict__ ip_xi, double* __restrict__ x) {
    constexpr int NEN = Shape<DIM, ORDER>::NEN;
    int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (k >= n) return;
    int eidx[3];
    el_index(g, cell[k], eidx);
    double xi[3] = {0.0, 0.0, 0.0}, N[NEN];
#pragma unroll
    for (int d = 0; d < DIM; d++) xi[d] = ip_xi[slot[k] * DIM + d];
    Shape<DIM, ORDER>::N(xi, N);
    double acc[3] = {0.0, 0.0, 0.0};
#pragma unroll
    for (int a = 0; a < NEN; a++)
#pragma unroll
        for (int d = 0; d < DIM; d++) acc[d] += N[a] * node_coord<DIM, ORDER>(g, eidx, a, d);
#pragma unroll
    for (int d = 0; d < DIM; d++) x[(int64_t)idx[k] * DIM + d] = acc[d];
}

uwg_geom pop_geom(const uwg_ctx* c) {
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

}  // namespace

extern "C" int uwg_pop_plan_escaped(uwg_ctx* c, int64_t np, const int32_t* owner, const int32_t* cell_offsets,
                                    const int32_t* cell_list, int64_t* np_new_h) {
    if (!c || np < 0 || !np_new_h || (np && (!owner || !cell_offsets || !cell_list)))
        return uwg_set_error(c, UWG_ERR_ARG, "uwg_pop_plan_escaped: bad argument");
    uwg_pop_free(c);
    std::vector<int32_t> ho, hf, hl;
    int rc = fetch_tables(c, np, owner, cell_offsets, cell_list, ho, hf, hl);
    if (rc) return rc;
    Replay R(np, (int32_t)c->n_el, ho, hf, hl);
    // _EscapedRoutine_Select (ascending scan), then removal from the highest index down
    std::vector<int64_t> esc;
    for (int64_t p = 0; p < np; p++)
        if (ho[p] < 0 || ho[p] >= c->n_el) esc.push_back(p);
    for (size_t k = esc.size(); k-- > 0;)
        if (!R.remove_index(esc[k])) return uwg_set_error(c, UWG_ERR_STATE, "escaped removal: cell tables inconsistent");
    uwg_pop* P = new uwg_pop();
    P->np_old = np;
    R.finish(*P);
    c->pop = P;
    *np_new_h = P->np_new;
    return UWG_OK;
}

extern "C" int uwg_pop_plan_pcdvc(uwg_ctx* c, int64_t np, const int32_t* owner, const int32_t* cell_offsets,
                                  const int32_t* cell_list, const double* ip_w, double split_threshold,
                                  double delete_threshold, int max_splits, int max_deletions, int64_t* np_new_h,
                                  int64_t* n_split_h, int64_t* n_deleted_h) {
    if (!c || np < 0 || !np_new_h || max_splits < 0 || max_deletions < 0 ||
        (np && (!owner || !cell_offsets || !cell_list || !ip_w)))
        return uwg_set_error(c, UWG_ERR_ARG, "uwg_pop_plan_pcdvc: bad argument");
    uwg_pop_free(c);
    std::vector<int32_t> ho, hf, hl;
    int rc = fetch_tables(c, np, owner, cell_offsets, cell_list, ho, hf, hl);
    if (rc) return rc;
    if ((int64_t)hl.size() != np) return uwg_set_error(c, UWG_ERR_STATE, "population control: particles outside the mesh");
    std::vector<double> w(np);
    if (np) UWG_CUDA(c, cudaMemcpy(w.data(), ip_w, sizeof(double) * np, cudaMemcpyDeviceToHost));
    // thresholds as the reference forms them: upperT = splitThreshold * 100 (P/swarm/_weights.py:112),
    // maxW = upT * cellVolume / 100.0 with the local cell volume 4 (2D) or 8 (3D) (PCDVC.c:578-579, 950-951)
    const double upT = split_threshold * 100., lowT = delete_threshold * 100.;
    const double vol = c->dim == 2 ? 4 : 8;
    const double maxW = upT * vol / 100.0, minW = lowT * vol / 100.0;
    Replay R(np, (int32_t)c->n_el, ho, hf, hl);
    int64_t n_split = 0, n_del = 0;
    std::vector<int64_t> splits;
    std::vector<int32_t> dels;
    for (int32_t cell = 0; cell < (int32_t)c->n_el; cell++) {
        const int32_t s0 = hf[cell], n = hf[cell + 1] - hf[cell];
        splits.clear();
        dels.clear();
        auto it = R.mod.find(cell);
        for (int32_t j = 0; j < n; j++) {
            const double wj = w[s0 + j];
            const int32_t idx = it == R.mod.end() ? hl[s0 + j] : it->second[j];
            if (wj > maxW) splits.push_back(j);
            if (wj < minW) dels.push_back(idx);
        }
        const int64_t ns = std::min<int64_t>(max_splits, (int64_t)splits.size());
        const int64_t nd = std::min<int64_t>(max_deletions, (int64_t)dels.size());
        if (ns == 0 && nd == 0) continue;
        for (int64_t k = 0; k < ns; k++) {
            const int32_t idx = R.list(cell)[splits[k]];
            R.append(cell, R.ident[idx], s0 + splits[k]);
        }
        // deleteList sorted by particle index, largest first (compare_indexOnCPU, PCDVC.c:296-304)
        std::sort(dels.begin(), dels.end(), [](int32_t a, int32_t b) { return a > b; });
        for (int64_t k = 0; k < nd; k++) {
            const int32_t p = dels[k];
            auto& L = R.list(cell);
            auto pos = std::find(L.begin(), L.end(), p);
            if (pos == L.end()) return uwg_set_error(c, UWG_ERR_STATE, "population control: cell tables inconsistent");
            *pos = L.back();
            L.pop_back();
            if (!R.remove_index(p)) return uwg_set_error(c, UWG_ERR_STATE, "population control: cell tables inconsistent");
        }
        n_split += ns;
        n_del += nd;
    }
    uwg_pop* P = new uwg_pop();
    P->np_old = np;
    R.finish(*P);
    c->pop = P;
    *np_new_h = P->np_new;
    if (n_split_h) *n_split_h = n_split;
    if (n_deleted_h) *n_deleted_h = n_del;
    return UWG_OK;
}

extern "C" int uwg_pop_apply(uwg_ctx* c, const double* ip_xi, const double* x_old, double* x_new, int32_t* owner_new,
                             int32_t* cell_offsets_new, int32_t* cell_list_new, int64_t* src_h) {
    if (!c || !c->pop) return uwg_set_error(c, UWG_ERR_STATE, "uwg_pop_apply: no pending plan");
    uwg_pop* P = (uwg_pop*)c->pop;
    const int64_t n = P->np_new, nn = (int64_t)P->new_index.size();
    if ((n && (!x_old || !x_new || !owner_new || !cell_list_new)) || !cell_offsets_new || (nn && !ip_xi))
        return uwg_set_error(c, UWG_ERR_ARG, "uwg_pop_apply: bad argument");
    int32_t *d_src = nullptr, *d_idx = nullptr, *d_cell = nullptr;
    int64_t* d_slot = nullptr;
    UWG_CUDA(c, cudaMallocAsync((void**)&d_src, sizeof(int32_t) * std::max<int64_t>(n, 1), c->stream));
    UWG_CUDA(c, cudaMallocAsync((void**)&d_idx, sizeof(int32_t) * std::max<int64_t>(nn, 1), c->stream));
    UWG_CUDA(c, cudaMallocAsync((void**)&d_cell, sizeof(int32_t) * std::max<int64_t>(nn, 1), c->stream));
    UWG_CUDA(c, cudaMallocAsync((void**)&d_slot, sizeof(int64_t) * std::max<int64_t>(nn, 1), c->stream));
    cudaError_t e = cudaSuccess;
    if (n) {
        e = cudaMemcpyAsync(d_src, P->src.data(), sizeof(int32_t) * n, cudaMemcpyHostToDevice, c->stream);
        if (e == cudaSuccess) e = cudaMemcpyAsync(owner_new, P->owner.data(), sizeof(int32_t) * n, cudaMemcpyHostToDevice, c->stream);
        if (e == cudaSuccess && !P->lst.empty())
            e = cudaMemcpyAsync(cell_list_new, P->lst.data(), sizeof(int32_t) * P->lst.size(), cudaMemcpyHostToDevice, c->stream);
        if (e == cudaSuccess) {
            k_pop_gather<<<nblk(n), 256, 0, c->stream>>>(n, c->dim, d_src, x_old, x_new);
            e = cudaGetLastError();
        }
    }
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(cell_offsets_new, P->off.data(), sizeof(int32_t) * P->off.size(), cudaMemcpyHostToDevice, c->stream);
    if (e == cudaSuccess && nn) {
        e = cudaMemcpyAsync(d_idx, P->new_index.data(), sizeof(int32_t) * nn, cudaMemcpyHostToDevice, c->stream);
        if (e == cudaSuccess) e = cudaMemcpyAsync(d_cell, P->new_cell.data(), sizeof(int32_t) * nn, cudaMemcpyHostToDevice, c->stream);
        if (e == cudaSuccess) e = cudaMemcpyAsync(d_slot, P->new_slot.data(), sizeof(int64_t) * nn, cudaMemcpyHostToDevice, c->stream);
        if (e == cudaSuccess) {
            uwg_geom g = pop_geom(c);
            if (c->dim == 2 && c->order == 1) k_pop_new_coords<2, 1><<<nblk(nn), 256, 0, c->stream>>>(g, nn, d_idx, d_cell, d_slot, ip_xi, x_new);
            else if (c->dim == 3 && c->order == 1) k_pop_new_coords<3, 1><<<nblk(nn), 256, 0, c->stream>>>(g, nn, d_idx, d_cell, d_slot, ip_xi, x_new);
            else if (c->dim == 2) k_pop_new_coords<2, 2><<<nblk(nn), 256, 0, c->stream>>>(g, nn, d_idx, d_cell, d_slot, ip_xi, x_new);
            else k_pop_new_coords<3, 2><<<nblk(nn), 256, 0, c->stream>>>(g, nn, d_idx, d_cell, d_slot, ip_xi, x_new);
            e = cudaGetLastError();
        }
    }
    if (src_h)
        for (int64_t i = 0; i < n; i++) src_h[i] = P->src[i];
    // the host vectors must outlive the copies
    cudaError_t e2 = cudaStreamSynchronize(c->stream);
    cudaFreeAsync(d_src, c->stream);
    cudaFreeAsync(d_idx, c->stream);
    cudaFreeAsync(d_cell, c->stream);
    cudaFreeAsync(d_slot, c->stream);
    uwg_pop_free(c);
    if (e != cudaSuccess) return uwg_set_error(c, UWG_ERR_CUDA, cudaGetErrorString(e));
    if (e2 != cudaSuccess) return uwg_set_error(c, UWG_ERR_CUDA, cudaGetErrorString(e2));
    return UWG_OK;
}
