// Context management and the remaining extern "C" entry points of libuwg.
//
//   L/ = src/underworld/libUnderworld/
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "uwg_ops.cuh"

int uwg_set_error(uwg_ctx* c, int code, const std::string& msg) {
    if (c) c->err = msg;
    return code;
}

extern "C" const char* uwg_last_error(const uwg_ctx* c) { return c ? c->err.c_str() : "null context"; }

static void* dmalloc(size_t bytes, bool* ok) {
    void* p = nullptr;
    if (cudaMalloc(&p, bytes ? bytes : 8) != cudaSuccess) { *ok = false; return nullptr; }
    return p;
}

extern "C" void uwg_ctx_destroy(uwg_ctx* c) {
    if (!c) return;
    cudaDeviceSynchronize();
    for (int d = 0; d < 3; d++) if (c->ax[d]) cudaFree(c->ax[d]);
    for (int l = 0; l < c->nlev; l++) {
        uwg_level& L = c->lev[l];
        if (l > 0) for (int d = 0; d < 3; d++) if (L.ax[d]) cudaFree(L.ax[d]);
        cudaFree(L.W64); cudaFree(L.W32); cudaFree(L.bc); cudaFree(L.diag64); cudaFree(L.diag32);
        if (L.cinv64) cudaFree(L.cinv64);
        if (L.tile_bc) cudaFree(L.tile_bc);
        if (L.Wdf) cudaFree(L.Wdf);
        for (int d = 0; d < 3; d++) if (L.h2inv[d]) cudaFree(L.h2inv[d]);
        if (L.cinv32) cudaFree(L.cinv32);
    }
    cudaFree(c->f); cudaFree(c->h); cudaFree(c->Shat); cudaFree(c->Mp); cudaFree(c->bcval);
    cudaFree(c->red);
    if (c->slcn_ws) cudaFree(c->slcn_ws);
    uwg_pop_free(c);
    if (c->q2_ke) cudaFree(c->q2_ke);
    if (c->q2_ke_df) cudaFree(c->q2_ke_df);
    if (c->cnn_flag) cudaFree(c->cnn_flag);
    if (c->red_host) cudaFreeHost(c->red_host);
    uwg_solver_free(c);
    delete c;
}

// Node coordinates per axis, CartesianGenerator_CalcGeom
// (L/StgDomain/Mesh/src/CartesianGenerator.c:2003-2036, contact depth 0).
static std::vector<double> axis_coords(int n_el_axis, int order, double mn, double mx) {
    int n = n_el_axis * order + 1;
    std::vector<double> v(n);
    double steps = mx - mn;
    for (int i = 0; i < n; i++) {
        if (i <= 0) v[i] = mn;
        else if (i >= n - 1) v[i] = mx;
        else v[i] = mn + ((double)i / (double)(n - 1)) * steps;
    }
    return v;
}

extern "C" int uwg_ctx_create(const uwg_mesh_desc* d, uwg_ctx** out) {
    if (!d || !out) return UWG_ERR_ARG;
    *out = nullptr;
    if (d->dim != 2 && d->dim != 3) return UWG_ERR_ARG;
    // Q1/dQ0 and Q2/dPc1, 2D and 3D
    bool q1 = d->order == 1 && d->porder == 0, q2 = d->order == 2 && d->porder == 1;
    if (!q1 && !q2) return UWG_ERR_ARG;
    for (int i = 0; i < d->dim; i++)
        if (d->res[i] < 1 || !(d->maxc[i] > d->minc[i])) return UWG_ERR_ARG;
    int dev_count = 0;
    if (cudaGetDeviceCount(&dev_count) != cudaSuccess || dev_count < 1) return UWG_ERR_CUDA;
    uwg_ctx* c = new uwg_ctx();
    memset(c->lev, 0, sizeof(c->lev));
    c->dim = d->dim;
    c->order = d->order;
    c->porder = d->porder;
    for (int i = 0; i < 3; i++) {
        c->res[i] = i < d->dim ? d->res[i] : 1;
        c->minc[i] = i < d->dim ? d->minc[i] : 0.0;
        c->maxc[i] = i < d->dim ? d->maxc[i] : 1.0;
        c->ax[i] = nullptr;
    }
    c->stream = 0;
    c->n_el = (int64_t)c->res[0] * c->res[1] * c->res[2];
    int64_t nn = 1;
    for (int i = 0; i < c->dim; i++) nn *= (int64_t)c->res[i] * c->order + 1;
    c->n_nodes = nn;
    c->n_vdof = nn * c->dim;
    c->nen = c->order == 2 ? (c->dim == 3 ? 27 : 9) : (c->dim == 3 ? 8 : 4);
    c->npn = c->porder == 1 ? (c->dim == 3 ? 4 : 3) : 1;
    c->n_pdof = c->n_el * c->npn;
    c->nq = c->order == 2 ? (c->dim == 3 ? 125 : 25) : (c->dim == 3 ? 27 : 9);
    c->dvc_res = 15;
    c->assembled = false;
    c->red_host = nullptr;
    bool ok = true;
    // finest axes and minimum separation (Mesh_HexType_GetMinimumSeparationGeneral,
    // L/StgDomain/Mesh/src/Mesh_HexType.c:275-332: the closest node pair of any
    // element; on a regular mesh an adjacent pair along one axis)
    double minsep = HUGE_VAL;
    std::vector<double> hax[3];
    for (int i = 0; i < c->dim; i++) {
        hax[i] = axis_coords(c->res[i], c->order, c->minc[i], c->maxc[i]);
        for (size_t k = 0; k + 1 < hax[i].size(); k++) {
            double dd = hax[i][k] - hax[i][k + 1];
            double m = std::sqrt(dd * dd);
            if (m < minsep) minsep = m;
        }
        c->ax[i] = (double*)dmalloc(sizeof(double) * hax[i].size(), &ok);
        if (ok) cudaMemcpy(c->ax[i], hax[i].data(), sizeof(double) * hax[i].size(), cudaMemcpyHostToDevice);
    }
    c->min_sep = minsep;
    // multigrid levels: halve while every axis is even (reference rule, L/.../_bsscr.py:73-91);
    // a Q2 context adds the Q1 mesh on the same elements as level 1
    const int q2lev = c->order == 2 ? 1 : 0;
    int nlev = 1;
    {
        int r[3] = {c->res[0], c->res[1], c->res[2]};
        while (nlev < UWG_MAXLEV) {
            bool even = true;
            for (int i = 0; i < c->dim; i++) even = even && (r[i] % 2 == 0);
            if (!even) break;
            for (int i = 0; i < c->dim; i++) r[i] /= 2;
            nlev++;
        }
    }
    nlev = std::min(nlev + q2lev, UWG_MAXLEV);
    c->nlev = nlev;
    for (int l = 0; l < nlev && ok; l++) {
        uwg_level& L = c->lev[l];
        L.order = (q2lev && l == 0) ? 2 : 1;
        L.nq = L.order == 2 ? (c->dim == 3 ? 125 : 25) : (c->dim == 3 ? 27 : 9);
        const int shift = q2lev ? std::max(l - 1, 0) : l;
        int64_t ne = 1, nnod = 1;
        for (int i = 0; i < 3; i++) {
            L.res[i] = i < c->dim ? (c->res[i] >> shift) : 1;
            ne *= L.res[i];
            if (i < c->dim) nnod *= (int64_t)L.res[i] * L.order + 1;
        }
        L.n_el = ne;
        L.n_nodes = nnod;
        L.n_dof = nnod * c->dim;
        for (int i = 0; i < 3; i++) {
            if (i >= c->dim) { L.ax[i] = nullptr; continue; }
            if (l == 0) { L.ax[i] = c->ax[i]; continue; }
            std::vector<double> v(L.res[i] + 1);
            for (int k = 0; k <= L.res[i]; k++) v[k] = hax[i][(size_t)k << l];
            L.ax[i] = (double*)dmalloc(sizeof(double) * v.size(), &ok);
            if (ok) cudaMemcpy(L.ax[i], v.data(), sizeof(double) * v.size(), cudaMemcpyHostToDevice);
        }
        for (int i = 0; i < 3; i++) {
            // 2/h per element along each axis in FP32, as the tiled FP32 apply forms it
            L.h2inv[i] = nullptr;
            if (i >= c->dim || L.order != 1) continue;
            std::vector<float> hv(L.res[i]);
            for (int k = 0; k < L.res[i]; k++) {
                double a = l == 0 ? hax[i][k] : hax[i][(size_t)k << l];
                double b = l == 0 ? hax[i][k + 1] : hax[i][(size_t)(k + 1) << l];
                hv[k] = 2.0f / (float)(b - a);
            }
            L.h2inv[i] = (float*)dmalloc(sizeof(float) * hv.size(), &ok);
            if (ok) cudaMemcpy(L.h2inv[i], hv.data(), sizeof(float) * hv.size(), cudaMemcpyHostToDevice);
        }
        L.W64 = (double*)dmalloc(sizeof(double) * L.nq * ne, &ok);
        L.W32 = (float*)dmalloc(sizeof(float) * L.nq * ne, &ok);
        L.bc = (uint8_t*)dmalloc(L.n_dof, &ok);
        L.diag64 = (double*)dmalloc(sizeof(double) * L.n_dof, &ok);
        L.diag32 = (float*)dmalloc(sizeof(float) * L.n_dof, &ok);
        if (ok) cudaMemset(L.bc, 0, L.n_dof);
        L.lmax64 = L.lmax32 = 1.0;
        L.cinv64 = nullptr;
        L.cinv32 = nullptr;
        if (l == nlev - 1) {
            if (L.n_dof > 4096) {
                ok = false;
            } else {
                L.cinv64 = (double*)dmalloc(sizeof(double) * L.n_dof * L.n_dof, &ok);
                L.cinv32 = (float*)dmalloc(sizeof(float) * L.n_dof * L.n_dof, &ok);
            }
        }
    }
    c->bc = c->lev[0].bc;
    // the pressure hierarchy ends at the first level of at most 512 cells (two unknowns
    // each below level 0): a dense solve there replaces the tiny, launch-bound levels
    c->pnlev = 1;
    while (c->pnlev < nlev && (c->pnlev < 2 || c->lev[c->pnlev - 1].n_el > 512)) c->pnlev++;
    c->f = (double*)dmalloc(sizeof(double) * c->n_vdof, &ok);
    c->bcval = (double*)dmalloc(sizeof(double) * c->n_vdof, &ok);
    c->h = (double*)dmalloc(sizeof(double) * c->n_pdof, &ok);
    c->Shat = (double*)dmalloc(sizeof(double) * c->n_el * c->npn * c->npn, &ok);
    c->Mp = (double*)dmalloc(sizeof(double) * c->n_pdof, &ok);
    c->red = dmalloc(4096 * sizeof(double), &ok);
    if (ok && cudaMallocHost((void**)&c->red_host, 4096 * sizeof(double)) != cudaSuccess) ok = false;
    if (ok) {
        cudaMemset(c->bcval, 0, sizeof(double) * c->n_vdof);
        cudaMemset(c->h, 0, sizeof(double) * c->n_pdof);
        cudaMemset(c->Mp, 0, sizeof(double) * c->n_pdof);
        cudaMemset(c->f, 0, sizeof(double) * c->n_vdof);
    }
    if (ok && c->order == 2 && uwg_q2_init(c) != UWG_OK) ok = false;
    if (!ok || cudaDeviceSynchronize() != cudaSuccess) {
        uwg_ctx_destroy(c);
        return UWG_ERR_CUDA;
    }
    *out = c;
    return UWG_OK;
}

extern "C" int uwg_set_stream(uwg_ctx* c, void* s) {
    if (!c) return UWG_ERR_ARG;
    c->stream = (cudaStream_t)s;
    return UWG_OK;
}

extern "C" int uwg_sync(uwg_ctx* c) {
    if (!c) return UWG_ERR_ARG;
    UWG_CUDA(c, cudaStreamSynchronize(c->stream));
    return UWG_OK;
}

extern "C" int uwg_mesh_sizes(const uwg_ctx* c, int64_t* s) {
    if (!c || !s) return UWG_ERR_ARG;
    s[0] = c->n_el; s[1] = c->n_nodes; s[2] = c->n_vdof; s[3] = c->n_pdof; s[4] = c->nen; s[5] = c->npn;
    s[6] = c->nlev;
    return UWG_OK;
}

extern "C" int uwg_mesh_axis(const uwg_ctx* c, int axis, double* out) {
    if (!c || !out || axis < 0 || axis >= c->dim) return UWG_ERR_ARG;
    size_t n = (size_t)c->res[axis] * c->order + 1;
    if (cudaMemcpy(out, c->ax[axis], sizeof(double) * n, cudaMemcpyDeviceToHost) != cudaSuccess) return UWG_ERR_CUDA;
    return UWG_OK;
}

extern "C" int uwg_set_bcs(uwg_ctx* c, const uint8_t* mask, const double* values) {
    if (!c || !mask) return uwg_set_error(c, UWG_ERR_ARG, "uwg_set_bcs: bad argument");
    UWG_CUDA(c, cudaMemcpyAsync(c->lev[0].bc, mask, c->n_vdof, cudaMemcpyDeviceToDevice, c->stream));
    if (values) {
        UWG_CUDA(c, cudaMemcpyAsync(c->bcval, values, sizeof(double) * c->n_vdof, cudaMemcpyDeviceToDevice, c->stream));
    } else {
        UWG_CUDA(c, cudaMemsetAsync(c->bcval, 0, sizeof(double) * c->n_vdof, c->stream));
    }
    for (int l = 0; l + 1 < c->nlev; l++) {
        int rc = uwg_ops_bc_coarsen(c, l);
        if (rc) return rc;
    }
    c->assembled = false;
    return UWG_OK;
}

__global__ void k_keep_bc(int64_t n, const uint8_t* bc, double* v) {
    int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i < n && !bc[i]) v[i] = 0.0;
}

extern "C" int uwg_assemble(uwg_ctx* c, int64_t np, const int32_t* off, const int32_t* list, const double* ip_xi,
                            const double* ip_w, const double* eta_p, const double* body_p, const double* lambda_p) {
    if (!c || !off || (np && (!list || !ip_xi || !ip_w || !eta_p)))
        return uwg_set_error(c, UWG_ERR_ARG, "uwg_assemble: bad argument");
    int rc = uwg_ops_assemble(c, off, list, ip_xi, ip_w, eta_p, body_p, lambda_p);
    if (rc) return rc;
    if (!lambda_p) UWG_CUDA(c, cudaMemsetAsync(c->Mp, 0, sizeof(double) * c->n_pdof, c->stream));
    c->compressible = lambda_p != nullptr;
    UWG_CUDA(c, cudaMemsetAsync(c->h, 0, sizeof(double) * c->n_pdof, c->stream));
    // Dirichlet lifting: f -= K_fb g, h -= G_b^T g  (StiffnessMatrix.c:627-678)
    k_keep_bc<<<(unsigned)((c->n_vdof + 255) / 256), 256, 0, c->stream>>>(c->n_vdof, c->bc, c->bcval);
    UWG_CUDA(c, cudaGetLastError());
    if ((rc = uwg_ops_applyK_lift(c, c->bcval, c->lev[0].diag64))) return rc;   // diag64 as scratch
    vk_axpy<double>(c->stream, c->n_vdof, -1.0, c->lev[0].diag64, c->f);
    vk_mask<double>(c->stream, c->n_vdof, c->bc, c->f);
    if ((rc = uwg_ops_applyGt_mode(c, c->bcval, c->Shat, 1))) return rc;           // Shat as scratch
    vk_axpy<double>(c->stream, c->n_pdof, -1.0, c->Shat, c->h);
    if ((rc = uwg_solver_setup(c))) return rc;
    UWG_CUDA(c, cudaStreamSynchronize(c->stream));
    c->assembled = true;
    c->asm_gen++;
    return UWG_OK;
}

__global__ void k_add_free(int64_t n, const uint8_t* bc, const double* df, double* f) {
    int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i < n && !bc[i]) f[i] += df[i];
}

extern "C" int uwg_add_force(uwg_ctx* c, const double* df) {
    if (!c || !df) return uwg_set_error(c, UWG_ERR_ARG, "uwg_add_force: bad argument");
    if (!c->assembled) return uwg_set_error(c, UWG_ERR_STATE, "uwg_add_force before uwg_assemble");
    k_add_free<<<(unsigned)((c->n_vdof + 255) / 256), 256, 0, c->stream>>>(c->n_vdof, c->bc, df, c->f);
    UWG_CUDA(c, cudaGetLastError());
    return UWG_OK;
}

// Continuity source term h_e[b] += sum_q w_q detJ src_q M_b(xi_q) over the PIC
// points of each element: VectorAssemblyTerm_NA__Fn on the pressure variable
// (L/Underworld/Utils/src/VectorAssemblyTerm_NA__Fn.cpp:143-202; N = the pressure
// basis, detJ from the velocity geometry), as P/systems/_stokes.py:284-288 adds
// it for fn_source.  One thread per element; elements are affine, so detJ is
// the product of the half-extents.  dPc1 bases: BilinearInnerElType.c:169-179,
// TrilinearInnerElType.c:202-216 (the same expressions, term for term).
template <int DIM>
__global__ void k_add_source(int64_t n_el, int order, int npn, int rx, int ry, const double* ax0, const double* ax1,
                             const double* ax2, const int32_t* off, const int32_t* list, const double* ip_xi,
                             const double* ip_w, const double* src_p, double* h) {
    int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (e >= n_el) return;
    int64_t ie[3] = {e % rx, (e / rx) % ry, DIM == 3 ? e / ((int64_t)rx * ry) : 0};
    const double* ax[3] = {ax0, ax1, ax2};
    double detJ = 1.0;
    for (int d = 0; d < DIM; d++) detJ *= 0.5 * (ax[d][order * ie[d] + order] - ax[d][order * ie[d]]);
    double acc[4] = {0.0, 0.0, 0.0, 0.0};
    for (int32_t s = off[e]; s < off[e + 1]; s++) {
        double fac = detJ * ip_w[s] * src_p[list[s]];
        const double* xi = ip_xi + (int64_t)s * DIM;
        if (npn == 1) {
            acc[0] += fac;
        } else if (DIM == 2) {
            double x = xi[0], y = xi[1];
            acc[0] += fac * (-x - 0.5 * y + 0.25);
            acc[1] += fac * (x - 0.5 * y + 0.25);
            acc[2] += fac * (y + 0.5);
        } else {
            double x = xi[0], y = xi[1], z = xi[DIM - 1], k = 1.0 / 9.0;
            acc[0] += fac * (k * (-4.0 * x - 20.0 * y + 12.0 * z + 3.0));
            acc[1] += fac * (k * (16.0 * x - 64.0 * y + 60.0 * z + 6.0));
            acc[2] += fac * (k * (36.0 * y - 36.0 * z));
            acc[3] += fac * (k * (-12.0 * x + 48.0 * y - 36.0 * z));
        }
    }
    for (int b = 0; b < npn; b++) h[e * npn + b] += acc[b];
}

extern "C" int uwg_add_source(uwg_ctx* c, const int32_t* off, const int32_t* list, const double* ip_xi,
                              const double* ip_w, const double* src_p) {
    if (!c || !off || !list || !ip_xi || !ip_w || !src_p) return uwg_set_error(c, UWG_ERR_ARG, "uwg_add_source: bad argument");
    if (!c->assembled) return uwg_set_error(c, UWG_ERR_STATE, "uwg_add_source before uwg_assemble");
    unsigned nb = (unsigned)((c->n_el + 127) / 128);
    if (c->dim == 3)
        k_add_source<3><<<nb, 128, 0, c->stream>>>(c->n_el, c->order, c->npn, c->res[0], c->res[1], c->ax[0], c->ax[1],
                                                   c->ax[2], off, list, ip_xi, ip_w, src_p, c->h);
    else
        k_add_source<2><<<nb, 128, 0, c->stream>>>(c->n_el, c->order, c->npn, c->res[0], c->res[1], c->ax[0], c->ax[1],
                                                   c->ax[0], off, list, ip_xi, ip_w, src_p, c->h);
    UWG_CUDA(c, cudaGetLastError());
    return UWG_OK;
}

extern "C" int uwg_element_matrices(uwg_ctx* c, int64_t el, double* Ke, double* fe, double* Ge, double* Se) {
    if (!c || el < 0 || el >= c->n_el) return uwg_set_error(c, UWG_ERR_ARG, "uwg_element_matrices: bad element");
    if (!c->assembled) return uwg_set_error(c, UWG_ERR_STATE, "element matrices before uwg_assemble");
    return uwg_ops_element_matrices(c, el, Ke, fe, Ge, Se);
}

extern "C" int uwg_apply_K64(uwg_ctx* c, int level, const double* x, double* y) {
    if (!c || !x || !y || level < 0 || level >= c->nlev) return uwg_set_error(c, UWG_ERR_ARG, "uwg_apply_K64: bad argument");
    if (!c->assembled) return uwg_set_error(c, UWG_ERR_STATE, "apply before uwg_assemble");
    return uwg_ops_applyK<double>(c, level, x, y);
}

// The operator of the mixed solve's refinement residuals (double-float on 3D Q2
// meshes with stored element matrices, else the FP64 apply).
extern "C" int uwg_apply_K_refine(uwg_ctx* c, const double* x, double* y) {
    if (!c || !x || !y) return uwg_set_error(c, UWG_ERR_ARG, "uwg_apply_K_refine: bad argument");
    if (!c->assembled) return uwg_set_error(c, UWG_ERR_STATE, "apply before uwg_assemble");
    return uwg_ops_applyK_refine(c, x, y);
}

extern "C" int uwg_apply_K32(uwg_ctx* c, int level, const float* x, float* y) {
    if (!c || !x || !y || level < 0 || level >= c->nlev) return uwg_set_error(c, UWG_ERR_ARG, "uwg_apply_K32: bad argument");
    if (!c->assembled) return uwg_set_error(c, UWG_ERR_STATE, "apply before uwg_assemble");
    return uwg_ops_applyK<float>(c, level, x, y);
}

extern "C" int uwg_apply_G(uwg_ctx* c, const double* p, double* y) {
    if (!c || !p || !y) return uwg_set_error(c, UWG_ERR_ARG, "uwg_apply_G: bad argument");
    return uwg_ops_applyG(c, p, y);
}

extern "C" int uwg_apply_Gt(uwg_ctx* c, const double* u, double* q) {
    if (!c || !u || !q) return uwg_set_error(c, UWG_ERR_ARG, "uwg_apply_Gt: bad argument");
    return uwg_ops_applyGt(c, u, q);
}
