// BSSCR Schur-complement Stokes solve on the GPU.
//
// Structure follows BSSCR_DRIVER_auglag with penalty 0
// (L/Solvers/KSPSolvers/src/BSSCR/auglag-driver-DGTGD.c:64-578):
//   1. velocity pre-solve      f~ = K^-1 f                         (:285-303)
//   2. h^ = h - G^T f~                                               (:309-310)
//   3. pressure solve          (C - G^T K^-1 G) p = h^  by FGMRES,   (:332-441)
//      preconditioned with the assembled Uzawa term S^ (PC "uw", preconditioner.c:164-174)
//   4. velocity back-solve     K u = f - G p                         (:494-532)
// The Krylov and multigrid kernels behind PETSc's KSP/PCMG are replaced by
// GPU-native ones: preconditioned CG on K (K is SPD once Dirichlet dofs are
// eliminated) with a geometric V-cycle (Chebyshev-Jacobi smoothing, Galerkin-
// exact coarse operators from coarsened quadrature weights, dense coarsest
// solve), and flexible GMRES on the Schur complement.  In mixed mode the
// velocity solves run in FP32 inside FP64 iterative refinement.
//
//   L/ = src/underworld/libUnderworld/
#include <chrono>
#include <cmath>
#include <cstring>
#include <vector>

#include <functional>

#include "uwg_ops.cuh"

namespace {

double now() {
    return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

template <typename T> struct LevelVecs { T *r, *d, *t, *b, *x; };

struct Work {
    bool ready = false;
    LevelVecs<double> v64[UWG_MAXLEV];
    LevelVecs<float> v32[UWG_MAXLEV];
    // finest-level Krylov vectors
    double *cg_r, *cg_z, *cg_p, *cg_q;       // FP64 PCG
    float *cg32_r, *cg32_z, *cg32_p, *cg32_q, *cg32_x, *cg32_b;
    double *ref_r, *ref_d;                    // refinement
    double *u_tmp, *u_tmp2;                   // velocity temps for the Schur apply
    double *ftil, *bvec;
    std::vector<double*> V, Z;                // FGMRES bases (pressure)
    double *p_tmp, *p_tmp2, *hhat;
    double* coef;                             // device coefficients
    int restart = 0;
    // pressure multigrid of the weighted BFBt preconditioner (FP32): one
    // unknown per cell on level 0, two (smooth, checkerboard) on coarser levels
    LevelVecs<float> pv[UWG_MAXLEV];
    float* pst[UWG_MAXLEV];                   // explicit cell stencils (uwg_pmg.cu layout)
    float* pdg[UWG_MAXLEV];                   // their diagonals
    float* pcinv = nullptr;                   // dense inverse of the coarsest level
    float* W0 = nullptr;                      // 1/sqrt(diag K) on level 0, 0 on Dirichlet dofs
    double Lmax[UWG_MAXLEV];
    float *pcg_r, *pcg_z, *pcg_p, *pcg_q, *bf_r, *bf_y, *bf_m, *bf_z, *bf_v1, *bf_v2;
    float *pf1 = nullptr, *pf2 = nullptr;    // level-0 scratch of the level-1 Galerkin apply
    int lsolve_its = 0;
    double t_pc = 0.0, t_schur = 0.0;          // seconds in the Schur preconditioner / operator
    // CUDA graphs of the V-cycles (captured at setup, replayed by the Krylov loops)
    cudaStream_t gstream = nullptr;
    cudaGraphExec_t g_v64 = nullptr, g_v32 = nullptr, g_pv = nullptr;
    cudaGraphExec_t g_lcg = nullptr;          // two CG iterations of the L-solve
    float* pcg_x = nullptr;                   // L-solve iterate (fixed buffer of the graph)
    double* lcg_s = nullptr;                  // L-solve scalars on the device
    double* lcg_h = nullptr;                  // pinned host mirror of lcg_s
    int g_deg = 0;
    int pdeg = 2, g_pdeg = 0;                  // pressure smoother degree (in use / captured)
    // pressure null space: even-cell / odd-cell indicator vectors, the constant, and
    // whether the checkerboard lies in the null space of G (every velocity dof on the walls fixed)
    double *ns_t = nullptr, *ns_v = nullptr, *ns_one = nullptr, *ns_tmp = nullptr;
    bool cb_null = false;
    bool const_null = false;   // the constant pressure lies in the null space of G
    // coarse-level correction of the Schur FGMRES (uwg_coarse.cu)
    double *cc_sinv = nullptr, *cc_tc = nullptr, *cc_zc = nullptr;
    int cc_agg = 0, cc_cap = 0;               // aggregate size of cc_sinv, its capacity (aggregates)
    int64_t cc_gen = -1;                      // assembly generation cc_sinv was built for
};

Work* work_of(uwg_ctx* c) {
    if (c->ws.empty()) c->ws.push_back(new Work());
    return (Work*)c->ws[0];
}

template <typename T> T* dalloc(uwg_ctx* c, int64_t n) {
    void* p = nullptr;
    if (cudaMalloc(&p, sizeof(T) * (n > 0 ? n : 1)) != cudaSuccess) return nullptr;
    c->ws.push_back(p);
    return (T*)p;
}

int work_init(uwg_ctx* c, int restart) {
    Work* w = work_of(c);
    if (w->ready && w->restart >= restart) return UWG_OK;
    int64_t nv = c->n_vdof, np = c->n_pdof;
    if (!w->ready) {
        for (int l = 0; l < c->nlev; l++) {
            int64_t n = c->lev[l].n_dof;
            w->v64[l] = {dalloc<double>(c, n), dalloc<double>(c, n), dalloc<double>(c, n), dalloc<double>(c, n), dalloc<double>(c, n)};
            w->v32[l] = {dalloc<float>(c, n), dalloc<float>(c, n), dalloc<float>(c, n), dalloc<float>(c, n), dalloc<float>(c, n)};
        }
        w->cg_r = dalloc<double>(c, nv); w->cg_z = dalloc<double>(c, nv);
        w->cg_p = dalloc<double>(c, nv); w->cg_q = dalloc<double>(c, nv);
        w->cg32_r = dalloc<float>(c, nv); w->cg32_z = dalloc<float>(c, nv);
        w->cg32_p = dalloc<float>(c, nv); w->cg32_q = dalloc<float>(c, nv); w->cg32_x = dalloc<float>(c, nv);
        w->cg32_b = dalloc<float>(c, nv);
        w->ref_r = dalloc<double>(c, nv); w->ref_d = dalloc<double>(c, nv);
        w->u_tmp = dalloc<double>(c, nv); w->u_tmp2 = dalloc<double>(c, nv);
        w->ftil = dalloc<double>(c, nv); w->bvec = dalloc<double>(c, nv);
        w->p_tmp = dalloc<double>(c, np); w->p_tmp2 = dalloc<double>(c, np); w->hhat = dalloc<double>(c, np);
        w->coef = dalloc<double>(c, 512);
        for (int l = 0; l < c->pnlev && c->porder == 0; l++) {   // the BFBt pressure multigrid is dQ0 only
            int64_t ne = uwg_pmg_ncomp(l) * c->lev[l].n_el;
            w->pv[l] = {dalloc<float>(c, ne), dalloc<float>(c, ne), dalloc<float>(c, ne), dalloc<float>(c, ne), dalloc<float>(c, ne)};
            w->pst[l] = dalloc<float>(c, uwg_pmg_stencil_size(c, l));
            w->pdg[l] = dalloc<float>(c, ne);
            w->Lmax[l] = 1.0;
            if (l == c->pnlev - 1) w->pcinv = dalloc<float>(c, ne * ne);
            if (!w->pst[l] || !w->pdg[l] || !w->pv[l].x) return uwg_set_error(c, UWG_ERR_CUDA, "out of device memory (pressure multigrid)");
        }
        w->W0 = dalloc<float>(c, nv);
        w->pcg_r = dalloc<float>(c, np); w->pcg_z = dalloc<float>(c, np);
        w->pcg_x = dalloc<float>(c, np);
        w->lcg_s = dalloc<double>(c, 16);
        if (!w->lcg_h && cudaMallocHost((void**)&w->lcg_h, sizeof(double) * 16) != cudaSuccess) w->lcg_h = nullptr;
        w->pcg_p = dalloc<float>(c, np); w->pcg_q = dalloc<float>(c, np);
        w->bf_r = dalloc<float>(c, np); w->bf_y = dalloc<float>(c, np);
        w->bf_m = dalloc<float>(c, np); w->bf_z = dalloc<float>(c, np);
        w->bf_v1 = dalloc<float>(c, nv); w->bf_v2 = dalloc<float>(c, nv);
        w->pf1 = dalloc<float>(c, np); w->pf2 = dalloc<float>(c, np);
        w->ns_t = dalloc<double>(c, np); w->ns_v = dalloc<double>(c, np); w->ns_one = dalloc<double>(c, np);
        w->ns_tmp = dalloc<double>(c, np);
    }
    while ((int)w->V.size() < restart + 1) w->V.push_back(dalloc<double>(c, np));
    while ((int)w->Z.size() < restart) w->Z.push_back(dalloc<double>(c, np));
    w->restart = restart;
    w->ready = true;
    for (double* p : w->V) if (!p) return uwg_set_error(c, UWG_ERR_CUDA, "out of device memory (solver workspace)");
    if (!w->coef) return uwg_set_error(c, UWG_ERR_CUDA, "out of device memory (solver workspace)");
    return UWG_OK;
}

// Deterministic probe vectors (power-iteration starts, the ||G|| estimate),
// filled on the device: x[i] = c0 + a sin(b i) + c (-1)^(i+1).  Dirichlet dofs
// are zeroed by the caller.
template <typename T>
__global__ void k_power_start(int64_t n, double c0, double a, double b, double cterm, T* x) {
    int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i < n) x[i] = (T)(c0 + a * sin(b * (double)i) + ((i & 1) ? cterm : -cterm));
}

// Host reductions through the context's pinned mirror.
template <typename T>
int dots(uwg_ctx* c, int64_t n, int k, const T* const* a, const T* const* b, double* out) {
    vk_dots<T>(c->stream, n, k, a, b, (double*)c->red);
    UWG_CUDA(c, cudaMemcpyAsync(c->red_host, c->red, sizeof(double) * k, cudaMemcpyDeviceToHost, c->stream));
    UWG_CUDA(c, cudaStreamSynchronize(c->stream));
    for (int j = 0; j < k; j++) out[j] = c->red_host[j];
    return UWG_OK;
}

template <typename T> double* diag_of(uwg_level& L);
template <> double* diag_of<double>(uwg_level& L) { return L.diag64; }

template <typename T> LevelVecs<T>& vecs(Work* w, int l);
template <> LevelVecs<double>& vecs<double>(Work* w, int l) { return w->v64[l]; }
template <> LevelVecs<float>& vecs<float>(Work* w, int l) { return w->v32[l]; }

template <typename T> const T* diagT(uwg_level& L);
template <> const double* diagT<double>(uwg_level& L) { return L.diag64; }
template <> const float* diagT<float>(uwg_level& L) { return L.diag32; }

// Chebyshev-Jacobi smoothing of K x = b on level l, `deg` applications
// (one operator apply and one fused update kernel per step).
template <typename T>
int chebyshev(uwg_ctx* c, int l, const T* b, T* x, int deg, bool x_zero) {
    uwg_level& L = c->lev[l];
    Work* w = work_of(c);
    LevelVecs<T>& v = vecs<T>(w, l);
    int64_t n = L.n_dof;
    cudaStream_t s = c->stream;
    double lmax = L.lmax64;
    double alpha = 0.1 * lmax, beta = 1.2 * lmax;
    double theta = 0.5 * (beta + alpha), delta = 0.5 * (beta - alpha);
    double sigma = theta / delta, rho = 1.0 / sigma;
    int rc;
    if (!x_zero && (rc = uwg_ops_applyK<T>(c, l, x, v.t))) return rc;
    vk_cheb<T>(s, n, b, x_zero ? nullptr : v.t, diagT<T>(L), (T)(1.0 / theta), (T)0, v.d, x, 1, x_zero ? 1 : 0);
    for (int i = 1; i < deg; i++) {
        if ((rc = uwg_ops_applyK<T>(c, l, x, v.t))) return rc;
        double rho1 = 1.0 / (2.0 * sigma - rho);
        vk_cheb<T>(s, n, b, v.t, diagT<T>(L), (T)(2.0 * rho1 / delta), (T)(rho1 * rho), v.d, x, 0, 0);
        rho = rho1;
    }
    return UWG_OK;
}

// V-cycle: x = M^-1 b on level l (x overwritten).
template <typename T>
int vcycle(uwg_ctx* c, int l, const T* b, T* x, int deg) {
    cudaStream_t s = c->stream;
    uwg_level& L = c->lev[l];
    int rc;
    if (l == c->nlev - 1) return uwg_ops_dense_solve<T>(c, l, b, x);
    Work* w = work_of(c);
    LevelVecs<T>& v = vecs<T>(w, l);
    LevelVecs<T>& vc = vecs<T>(w, l + 1);
    if ((rc = chebyshev<T>(c, l, b, x, deg, true))) return rc;
    if ((rc = uwg_ops_applyK<T>(c, l, x, v.t))) return rc;
    vk_axpby<T>(s, L.n_dof, (T)1, b, (T)-1, v.t);   // t = b - K x
    if ((rc = uwg_ops_restrict<T>(c, l + 1, v.t, vc.b))) return rc;
    if ((rc = vcycle<T>(c, l + 1, vc.b, vc.x, deg))) return rc;
    if ((rc = uwg_ops_prolong_add<T>(c, l + 1, vc.x, x))) return rc;
    return chebyshev<T>(c, l, b, x, deg, false);
}

template <typename T> cudaGraphExec_t graph_of(Work* w);
template <> cudaGraphExec_t graph_of<double>(Work* w) { return w->g_v64; }
template <> cudaGraphExec_t graph_of<float>(Work* w) { return w->g_v32; }
template <typename T> bool graph_buffers(Work* w, const T* b, const T* x);
template <> bool graph_buffers<double>(Work* w, const double* b, const double* x) { return b == w->cg_r && x == w->cg_z; }
template <> bool graph_buffers<float>(Work* w, const float* b, const float* x) { return b == w->cg32_r && x == w->cg32_z; }

// Finest-level V-cycle: the captured graph when the buffers match, else launched directly.
template <typename T>
int run_vcycle(uwg_ctx* c, const T* b, T* x, int deg) {
    Work* w = work_of(c);
    cudaGraphExec_t g = graph_of<T>(w);
    if (g && deg == w->g_deg && graph_buffers<T>(w, b, x)) {
        UWG_CUDA(c, cudaGraphLaunch(g, c->stream));
        return UWG_OK;
    }
    return vcycle<T>(c, 0, b, x, deg);
}

// Preconditioned CG on the finest level: x (in/out), stops at ||r|| <= tol*||b||
// (tol relative to bnorm passed in).  Returns iterations or negative error.
template <typename T>
int pcg(uwg_ctx* c, const T* b, T* x, double bnorm, double tol, int maxit, int deg, T* r, T* z, T* p, T* q,
        bool x_zero, int* its) {
    cudaStream_t s = c->stream;
    int64_t n = c->n_vdof;
    int rc;
    *its = 0;
    if (bnorm == 0.0) { vk_zero<T>(s, n, x); return UWG_OK; }
    if (x_zero) { vk_zero<T>(s, n, x); vk_copy<T>(s, n, b, r); }
    else {
        if ((rc = uwg_ops_applyK<T>(c, 0, x, q))) return rc;
        vk_copy<T>(s, n, b, r);
        vk_axpy<T>(s, n, (T)-1, q, r);
    }
    if ((rc = run_vcycle<T>(c, r, z, deg))) return rc;
    vk_copy<T>(s, n, z, p);
    double d2[2];
    const T* a2[2] = {r, r};
    const T* b2[2] = {z, r};
    if ((rc = dots<T>(c, n, 2, a2, b2, d2))) return rc;
    double rz = d2[0];
    if (!std::isfinite(bnorm) || !std::isfinite(d2[1]))
        return uwg_set_error(c, UWG_ERR_NAN, "velocity CG: non-finite right-hand side or residual");
    if (std::sqrt(d2[1]) <= tol * bnorm) return UWG_OK;
    for (int it = 1; it <= maxit; it++) {
        if ((rc = uwg_ops_applyK<T>(c, 0, p, q))) return rc;
        double pq;
        const T* a1[1] = {p};
        const T* b1[1] = {q};
        if ((rc = dots<T>(c, n, 1, a1, b1, &pq))) return rc;
        if (!std::isfinite(pq) || pq <= 0.0) {
            *its = it;
            return uwg_set_error(c, std::isfinite(pq) ? UWG_ERR_NOT_CONVERGED : UWG_ERR_NAN,
                                 "velocity CG breakdown (p.Kp = " + std::to_string(pq) + ")");
        }
        double alpha = rz / pq;
        vk_axpy<T>(s, n, (T)alpha, p, x);
        vk_axpy<T>(s, n, (T)-alpha, q, r);
        if ((rc = run_vcycle<T>(c, r, z, deg))) return rc;
        if ((rc = dots<T>(c, n, 2, a2, b2, d2))) return rc;
        *its = it;
        if (!std::isfinite(d2[1])) return uwg_set_error(c, UWG_ERR_NAN, "non-finite residual in velocity CG");
        if (std::sqrt(d2[1]) <= tol * bnorm) return UWG_OK;
        if (!(d2[0] > 0.0) || !std::isfinite(d2[0]))
            return uwg_set_error(c, std::isfinite(d2[0]) ? UWG_ERR_NOT_CONVERGED : UWG_ERR_NAN,
                                 "velocity CG: preconditioned residual r.z = " + std::to_string(d2[0]) +
                                 " at ||r||/||b|| = " + std::to_string(std::sqrt(d2[1]) / bnorm));
        double beta = d2[0] / rz;
        rz = d2[0];
        vk_axpby<T>(s, n, (T)1, z, (T)beta, p);
    }
    return uwg_set_error(c, UWG_ERR_NOT_CONVERGED, "velocity CG reached its iteration cap");
}

struct SolveCfg {
    bool mixed;
    double inner_rtol;
    int max_inner;
    int deg;
    int schur_pc;
    double schur_pc_rtol;
    bool relax;
    int schur_pc_its;   // > 0: fixed CG iterations per pressure-Laplacian solve (rtol ignored)
    int cc_agg = 0;     // > 0: coarse-level correction with this aggregate size (Sc^-1 built)
    double cc_rtol = 1e-2;
};

int bfbt(uwg_ctx* c, const double* r, double* z, double rtol, int its);

// x = A^-1 b for the velocity operator A = PKP + (I-P), FP64 result.
// x holds the initial guess unless x_zero.  Returns iterations through *its.
int velocity_solve(uwg_ctx* c, const SolveCfg& cfg, const double* b, double* x, bool x_zero, int* its,
                   int* refine_steps) {
    Work* w = work_of(c);
    cudaStream_t s = c->stream;
    int64_t n = c->n_vdof;
    double bn;
    const double* ab[1] = {b};
    int rc = dots<double>(c, n, 1, ab, ab, &bn);
    if (rc) return rc;
    bn = std::sqrt(bn);
    *its = 0;
    if (!cfg.mixed)
        return pcg<double>(c, b, x, bn, cfg.inner_rtol, cfg.max_inner, cfg.deg, w->cg_r, w->cg_z, w->cg_p,
                           w->cg_q, x_zero, its);
    // FP64 iterative refinement around FP32 PCG
    if (x_zero) vk_zero<double>(s, n, x);
    if (bn == 0.0) return UWG_OK;
    for (int step = 0; step < 30; step++) {
        vk_copy<double>(s, n, b, w->ref_r);
        if (step > 0 || !x_zero) {   // from a zero start the first residual is b itself
            if ((rc = uwg_ops_applyK_refine(c, x, w->ref_d))) return rc;
            vk_axpy<double>(s, n, -1.0, w->ref_d, w->ref_r);
        }
        double rn;
        const double* ar[1] = {w->ref_r};
        if ((rc = dots<double>(c, n, 1, ar, ar, &rn))) return rc;
        rn = std::sqrt(rn);
        if (!std::isfinite(rn)) return uwg_set_error(c, UWG_ERR_NAN, "non-finite residual in refinement");
        if (rn <= cfg.inner_rtol * bn) return UWG_OK;
        if (refine_steps) (*refine_steps)++;
        vk_convert<double, float>(s, n, w->ref_r, w->cg32_b);
        // the FP32 correction only needs a few digits; ask for 1e-5 of this residual
        double inner = std::max(1e-5, 0.5 * cfg.inner_rtol * bn / rn);
        int it32 = 0;
        rc = pcg<float>(c, w->cg32_b, w->cg32_x, rn, inner, cfg.max_inner, cfg.deg, w->cg32_r, w->cg32_z,
                        w->cg32_p, w->cg32_q, true, &it32);
        *its += it32;
        if (rc && rc != UWG_ERR_NOT_CONVERGED) return rc;
        vk_convert<float, double>(s, n, w->cg32_x, w->ref_d);
        vk_axpy<double>(s, n, 1.0, w->ref_d, x);
    }
    return uwg_set_error(c, UWG_ERR_NOT_CONVERGED, "velocity refinement did not converge");
}


// ---------------------------------------------------------------------------
// Weighted BFBt Schur preconditioner (scaled BFBt, May & Moresi, PEPI 2008,
// with the sqrt-diagonal weight of w-BFBt, Rudi et al., SISC 2017):
//   S^-1 ~ L^-1 (G^T W K W G) L^-1,  L = G^T W G,  W = diag(K)^-1/2.
// The square-root weight narrows the coefficient range of L (1e5 viscosity
// contrast -> ~300), which both improves the preconditioner and makes L easy
// for a cell-centred multigrid.  All of it runs in FP32: it is a
// preconditioner inside flexible GMRES, whose residuals stay FP64.
// ---------------------------------------------------------------------------
// y = A_l x on pressure-multigrid level l (level 0 in 3D without its stencil)
int papply(uwg_ctx* c, int l, const float* x, float* y) {
    Work* w = work_of(c);
    if (l == 0 && c->dim == 3) return uwg_pmg_apply0_mf(c, w->W0, x, y);
    if (l == 1 && c->pnlev >= 3) {
        // A_1 x = P^T (A_0 (P x)): the Galerkin product itself, applied through level 0.
        // Its stored stencil (smooth-checkerboard block, 206 coefficients per cell) costs
        // three times the bytes of the prolongation, level-0 apply and restriction.
        int rc;
        UWG_CUDA(c, cudaMemsetAsync(w->pf1, 0, sizeof(float) * c->lev[0].n_el, c->stream));
        if ((rc = uwg_pmg_prolong_add(c, 1, x, w->pf1))) return rc;
        if ((rc = papply(c, 0, w->pf1, w->pf2))) return rc;
        return uwg_pmg_restrict(c, 1, w->pf2, y);
    }
    return uwg_pmg_apply(c, l, w->pst[l], x, y);
}

int cheb_L(uwg_ctx* c, int l, const float* b, float* x, int deg, bool x_zero) {
    Work* w = work_of(c);
    LevelVecs<float>& v = w->pv[l];
    int64_t n = uwg_pmg_ncomp(l) * c->lev[l].n_el;
    cudaStream_t s = c->stream;
    double lmax = w->Lmax[l];
    double alpha = 0.1 * lmax, beta = 1.2 * lmax;
    double theta = 0.5 * (beta + alpha), delta = 0.5 * (beta - alpha);
    double sigma = theta / delta, rho = 1.0 / sigma;
    int rc;
    if (!x_zero && (rc = papply(c, l, x, v.t))) return rc;
    vk_cheb<float>(s, n, b, x_zero ? nullptr : v.t, w->pdg[l], (float)(1.0 / theta), 0.f, v.d, x, 1, x_zero ? 1 : 0);
    for (int i = 1; i < deg; i++) {
        if ((rc = papply(c, l, x, v.t))) return rc;
        double rho1 = 1.0 / (2.0 * sigma - rho);
        vk_cheb<float>(s, n, b, v.t, w->pdg[l], (float)(2.0 * rho1 / delta), (float)(rho1 * rho), v.d, x, 0, 0);
        rho = rho1;
    }
    return UWG_OK;
}

int pvcycle(uwg_ctx* c, int l, const float* b, float* x) {
    Work* w = work_of(c);
    cudaStream_t s = c->stream;
    int64_t n = uwg_pmg_ncomp(l) * c->lev[l].n_el;
    int rc;
    if (l == c->pnlev - 1) return uwg_ops_dense_mv32(c, n, w->pcinv, b, x);
    LevelVecs<float>& v = w->pv[l];
    LevelVecs<float>& vc = w->pv[l + 1];
    if ((rc = cheb_L(c, l, b, x, w->pdeg, true))) return rc;
    if ((rc = papply(c, l, x, v.t))) return rc;
    vk_axpby<float>(s, n, 1.f, b, -1.f, v.t);
    if ((rc = uwg_pmg_restrict(c, l + 1, v.t, vc.b))) return rc;
    if ((rc = pvcycle(c, l + 1, vc.b, vc.x))) return rc;
    if ((rc = uwg_pmg_prolong_add(c, l + 1, vc.x, x))) return rc;
    return cheb_L(c, l, b, x, w->pdeg, false);
}

int run_pvcycle(uwg_ctx* c, const float* b, float* x) {
    Work* w = work_of(c);
    if (w->g_pv && w->g_pdeg == w->pdeg && b == w->pcg_r && x == w->pcg_z) {
        UWG_CUDA(c, cudaGraphLaunch(w->g_pv, c->stream));
        return UWG_OK;
    }
    return pvcycle(c, 0, b, x);
}

// Capture `body` (kernels only, no host synchronisation) into an executable graph.
int capture(uwg_ctx* c, cudaGraphExec_t* out, const std::function<int()>& body) {
    Work* w = work_of(c);
    if (*out) { cudaGraphExecDestroy(*out); *out = nullptr; }
    if (!w->gstream) UWG_CUDA(c, cudaStreamCreateWithFlags(&w->gstream, cudaStreamNonBlocking));
    cudaStream_t saved = c->stream;
    UWG_CUDA(c, cudaStreamSynchronize(saved));
    c->stream = w->gstream;
    cudaError_t e = cudaStreamBeginCapture(w->gstream, cudaStreamCaptureModeThreadLocal);
    if (e != cudaSuccess) { c->stream = saved; return uwg_set_error(c, UWG_ERR_CUDA, cudaGetErrorString(e)); }
    int rc = body();
    cudaGraph_t g = nullptr;
    e = cudaStreamEndCapture(w->gstream, &g);
    c->stream = saved;
    if (rc) { if (g) cudaGraphDestroy(g); return rc; }
    if (e != cudaSuccess) return uwg_set_error(c, UWG_ERR_CUDA, std::string("graph capture: ") + cudaGetErrorString(e));
    e = cudaGraphInstantiate(out, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) return uwg_set_error(c, UWG_ERR_CUDA, std::string("graph instantiate: ") + cudaGetErrorString(e));
    return UWG_OK;
}

int capture_lcg(uwg_ctx* c);

int capture_cycles(uwg_ctx* c, int deg) {
    Work* w = work_of(c);
    int rc;
    if ((rc = capture(c, &w->g_v64, [&]() { return vcycle<double>(c, 0, w->cg_r, w->cg_z, deg); }))) return rc;
    if ((rc = capture(c, &w->g_v32, [&]() { return vcycle<float>(c, 0, w->cg32_r, w->cg32_z, deg); }))) return rc;
    if (c->porder == 0) {
        if ((rc = capture(c, &w->g_pv, [&]() { return pvcycle(c, 0, w->pcg_r, w->pcg_z); }))) return rc;
        if ((rc = capture_lcg(c))) return rc;
    }
    w->g_deg = deg;
    w->g_pdeg = w->pdeg;
    return UWG_OK;
}

// L-solve CG with its scalars on the device, so that iterations need no host
// round trip: S[4..5] / S[6..7] hold (r.z, r.r) of alternate iterations,
// S[2] holds p.q, S[9] flags a breakdown (p.q <= 0).
__global__ void k_lcg_step1(int64_t n, double* S, int rz_old, const float* p, const float* q, float* x, float* r) {
    __shared__ float al;
    __shared__ int ok;
    if (threadIdx.x == 0) {
        double pq = S[2];
        ok = pq > 0.0 && S[9] == 0.0;
        al = ok ? (float)(S[rz_old] / pq) : 0.f;
        if (!ok && blockIdx.x == 0) S[9] = 1.0;
    }
    __syncthreads();
    if (!ok) return;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        x[i] += al * p[i];
        r[i] -= al * q[i];
    }
}
__global__ void k_lcg_step2(int64_t n, const double* S, int rz_old, int rz_new, const float* z, float* p) {
    __shared__ float be;
    __shared__ int ok;
    if (threadIdx.x == 0) {
        ok = S[9] == 0.0;
        be = ok ? (float)(S[rz_new] / S[rz_old]) : 0.f;
    }
    __syncthreads();
    if (!ok) return;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        p[i] = z[i] + be * p[i];
}

// one CG iteration: old (r.z) in S[rz_old], new (r.z, r.r) into S[rz_new], S[rz_new + 1]
int lcg_iteration(uwg_ctx* c, int rz_old, int rz_new) {
    Work* w = work_of(c);
    cudaStream_t s = c->stream;
    int64_t n = c->n_pdof;
    unsigned nb = (unsigned)std::min<int64_t>((n + 255) / 256, 152 * 8);
    int rc;
    float *r = w->pcg_r, *z = w->pcg_z, *p = w->pcg_p, *q = w->pcg_q;
    if ((rc = papply(c, 0, p, q))) return rc;
    const float* a1[1] = {p};
    const float* b1[1] = {q};
    vk_dots<float>(s, n, 1, a1, b1, w->lcg_s + 2);
    k_lcg_step1<<<nb, 256, 0, s>>>(n, w->lcg_s, rz_old, p, q, w->pcg_x, r);
    if ((rc = pvcycle(c, 0, r, z))) return rc;
    const float* a2[2] = {r, r};
    const float* b2[2] = {z, r};
    vk_dots<float>(s, n, 2, a2, b2, w->lcg_s + rz_new);
    k_lcg_step2<<<nb, 256, 0, s>>>(n, w->lcg_s, rz_old, rz_new, z, p);
    UWG_CUDA(c, cudaGetLastError());
    return UWG_OK;
}

int capture_lcg(uwg_ctx* c) {
    Work* w = work_of(c);
    return capture(c, &w->g_lcg, [&]() {
        int rc = lcg_iteration(c, 4, 6);
        return rc ? rc : lcg_iteration(c, 6, 4);
    });
}

// x = L^-1 b by multigrid-preconditioned CG from zero, to rtol (FP32 vectors,
// FP64 reductions); convergence is checked every second iteration.
int lsolve(uwg_ctx* c, const float* b, float* x, double rtol, int maxit) {
    Work* w = work_of(c);
    cudaStream_t s = c->stream;
    int64_t n = c->n_pdof;
    int rc;
    if (!w->g_lcg || !w->lcg_h || w->g_pdeg != w->pdeg) return uwg_set_error(c, UWG_ERR_CUDA, "L-solve graph missing");
    float *r = w->pcg_r, *z = w->pcg_z, *p = w->pcg_p;
    vk_zero<float>(s, n, w->pcg_x);
    vk_copy<float>(s, n, b, r);
    if ((rc = run_pvcycle(c, r, z))) return rc;
    vk_copy<float>(s, n, z, p);
    UWG_CUDA(c, cudaMemsetAsync(w->lcg_s, 0, sizeof(double) * 16, s));
    const float* a2[2] = {r, r};
    const float* b2[2] = {z, r};
    vk_dots<float>(s, n, 2, a2, b2, w->lcg_s + 4);
    UWG_CUDA(c, cudaMemcpyAsync(w->lcg_h, w->lcg_s, sizeof(double) * 16, cudaMemcpyDeviceToHost, s));
    UWG_CUDA(c, cudaStreamSynchronize(s));
    double bn = std::sqrt(w->lcg_h[5]);
    if (bn > 0.0) {
        for (int it = 0; it < maxit; it += 2) {
            UWG_CUDA(c, cudaGraphLaunch(w->g_lcg, s));
            w->lsolve_its += 2;
            if (!(rtol > 0.0)) continue;   // fixed iterations: no host round trip (breakdowns stop on the device)
            UWG_CUDA(c, cudaMemcpyAsync(w->lcg_h, w->lcg_s, sizeof(double) * 16, cudaMemcpyDeviceToHost, s));
            UWG_CUDA(c, cudaStreamSynchronize(s));
            if (w->lcg_h[9] != 0.0 || !(std::sqrt(w->lcg_h[5]) > rtol * bn)) break;
        }
    }
    vk_copy<float>(s, n, w->pcg_x, x);
    return UWG_OK;   // a preconditioner: an inexact solve is acceptable
}

// ---------------------------------------------------------------------------
// Pressure null space (KSPBuildPressure_{Const,CB}_Nullspace_BSSCR and
// KSPRemovePressureNullspace_BSSCR, L/Solvers/KSPSolvers/src/BSSCR/
// ksp_pressure_nullspace.c:28-183).  Mode 1 is the constant vector; mode 2 is
// the pair of indicator vectors of the even cells (i+j+k even) and the odd
// cells, whose span holds both the constant and the checkerboard.  A vector
// is removed only when it lies in the null space of G:
// ||G t|| / ||t|| < nstol ||G||_inf with nstol = 1e-7 (BSSCR.c:428).
// ---------------------------------------------------------------------------
__global__ void k_ns_fill(int64_t n_el, int npn, int rx, int ry, double* t, double* v, double* one) {
    int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n_el * npn) return;
    int64_t e = i / npn;
    int64_t ex = e % rx, ey = (e / rx) % ry, ez = e / ((int64_t)rx * ry);
    bool even = ((ex + ey + ez) & 1) == 0;
    t[i] = even ? 1.0 : 0.0;
    v[i] = even ? 0.0 : 1.0;
    one[i] = 1.0;   // all pressure coefficients 1 is p = 1 for dQ0 and for dPc1 (its basis sums to 1)
}

int ns_fill(uwg_ctx* c) {
    Work* w = work_of(c);
    int64_t n = c->n_el * c->npn;
    k_ns_fill<<<(unsigned)((n + 255) / 256), 256, 0, c->stream>>>(c->n_el, c->npn, c->res[0], c->res[1], w->ns_t,
                                                                   w->ns_v, w->ns_one);
    UWG_CUDA(c, cudaGetLastError());
    return UWG_OK;
}

// ||G||_inf, the largest absolute row sum of the assembled gradient (MatNorm(G,
// NORM_INFINITY) at auglag-driver-DGTGD.c:410).  Q1/dQ0: an interior velocity row
// of component i couples to 2^dim cells with entries prod_{d != i} h_d / 2 (the
// closed form of k_gradG_nodes).  Q2/dPc1: estimated as ||G z|| / ||z|| for a
// fixed z, which is only used in the two threshold tests below.
int g_norm_inf(uwg_ctx* c, double* out) {
    Work* w = work_of(c);
    cudaStream_t s = c->stream;
    int rc;
    if (c->order == 1) {
        double hmax[3] = {1.0, 1.0, 1.0};
        for (int d = 0; d < c->dim; d++) {
            std::vector<double> ax(c->res[d] + 1);
            UWG_CUDA(c, cudaMemcpyAsync(ax.data(), c->ax[d], sizeof(double) * ax.size(), cudaMemcpyDeviceToHost, s));
            UWG_CUDA(c, cudaStreamSynchronize(s));
            hmax[d] = 0.0;
            for (int i = 0; i < c->res[d]; i++) hmax[d] = std::max(hmax[d], ax[i + 1] - ax[i]);
        }
        double best = 0.0;
        for (int i = 0; i < c->dim; i++) {
            double g = (double)(1 << c->dim);
            for (int d = 0; d < c->dim; d++)
                if (d != i) g *= 0.5 * hmax[d];
            best = std::max(best, g);
        }
        *out = best;
        return UWG_OK;
    }
    int64_t np = c->n_pdof;
    k_power_start<double><<<(unsigned)((np + 255) / 256), 256, 0, s>>>(np, 0.0, 1.0, 1.37, 0.3, w->ns_tmp);
    if ((rc = uwg_ops_applyG(c, w->ns_tmp, w->u_tmp))) return rc;
    double d[2];
    const double* a1[1] = {w->u_tmp};
    if ((rc = dots<double>(c, c->n_vdof, 1, a1, a1, d))) return rc;
    const double* a2[1] = {w->ns_tmp};
    if ((rc = dots<double>(c, np, 1, a2, a2, d + 1))) return rc;
    *out = d[1] > 0.0 ? std::sqrt(d[0] / d[1]) : 1.0;
    return UWG_OK;
}

// Does t lie in the null space of G (free rows)?
int ns_test(uwg_ctx* c, const double* t, double gnorm, bool* in_ns) {
    Work* w = work_of(c);
    int rc;
    if ((rc = uwg_ops_applyG(c, t, w->u_tmp))) return rc;   // Dirichlet rows are zero
    double d[2];
    const double* a1[1] = {w->u_tmp};
    if ((rc = dots<double>(c, c->n_vdof, 1, a1, a1, d))) return rc;
    const double* a2[1] = {t};
    if ((rc = dots<double>(c, c->n_pdof, 1, a2, a2, d + 1))) return rc;
    *in_ns = d[1] > 0.0 && std::sqrt(d[0] / d[1]) < 1e-7 * gnorm;
    return UWG_OK;
}

// x -= (t.x / t.t) t
int ns_project(uwg_ctx* c, const double* t, double* x) {
    double d[2];
    const double* a[2] = {t, t};
    const double* b[2] = {x, t};
    int rc = dots<double>(c, c->n_pdof, 2, a, b, d);
    if (rc) return rc;
    if (d[1] > 0.0) vk_axpy<double>(c->stream, c->n_pdof, -d[0] / d[1], t, x);
    return UWG_OK;
}

// z = -BFBt(r): the sign makes it approximate the inverse of C - G^T K^-1 G
int bfbt(uwg_ctx* c, const double* r, double* z, double rtol, int its) {
    Work* w = work_of(c);
    cudaStream_t s = c->stream;
    int64_t np = c->n_pdof, nv = c->n_vdof;
    int rc;
    if (w->cb_null) {
        // both null modes out of the input, so that the L-solves see consistent right-hand sides
        vk_copy<double>(s, np, r, w->ns_tmp);
        if ((rc = ns_project(c, w->ns_t, w->ns_tmp)) || (rc = ns_project(c, w->ns_v, w->ns_tmp))) return rc;
        r = w->ns_tmp;
    }
    const int maxit = its > 0 ? its : 200;
    if (its > 0) rtol = 0.0;   // a fixed number of iterations: flexible GMRES accepts the varying operator
    vk_convert<double, float>(s, np, r, w->bf_r);
    if ((rc = lsolve(c, w->bf_r, w->bf_y, rtol, maxit))) return rc;
    if ((rc = uwg_ops_G32(c, 0, w->W0, w->bf_y, w->bf_v1))) return rc;             // W G y
    if ((rc = uwg_ops_applyK<float>(c, 0, w->bf_v1, w->bf_v2))) return rc;         // K W G y
    vk_pointwise_mul_mask(s, nv, w->W0, w->bf_v2);                                  // W K W G y
    if ((rc = uwg_ops_Gt32(c, 0, w->bf_v2, w->bf_m))) return rc;
    if ((rc = lsolve(c, w->bf_m, w->bf_z, rtol, maxit))) return rc;
    vk_convert<float, double>(s, np, w->bf_z, z);
    vk_scale<double>(s, np, -1.0, z);
    // Null modes of S in z are arbitrary (L is singular on them) and S removes them
    // again; left in, a direction that is almost a pure null mode would give the
    // flexible GMRES a zero pivot near convergence.
    if (w->cb_null) {
        if ((rc = ns_project(c, w->ns_t, z)) || (rc = ns_project(c, w->ns_v, z))) return rc;
    } else if (w->const_null && (rc = ns_project(c, w->ns_one, z))) {
        return rc;
    }
    return UWG_OK;
}

int bfbt_setup(uwg_ctx* c) {
    Work* w = work_of(c);
    cudaStream_t s = c->stream;
    int rc;
    if ((rc = uwg_ops_winv(c, 0, w->W0))) return rc;
    for (int l = 0; l < c->pnlev; l++) {
        if ((rc = uwg_pmg_stencil(c, l, w->W0, l ? w->pst[l - 1] : nullptr, w->pst[l]))) return rc;
        if ((rc = uwg_pmg_diag(c, l, w->pst[l], w->pdg[l]))) return rc;
        if (l == c->pnlev - 1) break;
        // largest eigenvalue of D^-1 A by power iteration (Chebyshev interval)
        int64_t n = uwg_pmg_ncomp(l) * c->lev[l].n_el;
        LevelVecs<float>& v = w->pv[l];
        k_power_start<float><<<(unsigned)((n + 255) / 256), 256, 0, s>>>(n, 1.0, 0.41, 1.37, 0.3, v.x);
        double lam = 1.0;
        for (int it = 0; it < 30; it++) {
            if ((rc = papply(c, l, v.x, v.t))) return rc;
            vk_pointwise_div<float>(s, n, v.t, w->pdg[l], v.d);
            double d2[2];
            const float* a[2] = {v.d, v.x};
            if ((rc = dots<float>(c, n, 2, a, a, d2))) return rc;
            if (d2[0] <= 0.0 || d2[1] <= 0.0) break;
            lam = std::sqrt(d2[0] / d2[1]);
            vk_copy<float>(s, n, v.d, v.x);
            vk_scale<float>(s, n, (float)(1.0 / std::sqrt(d2[0])), v.x);
        }
        w->Lmax[l] = lam;
    }
    return uwg_pmg_dense_inverse(c, c->pnlev - 1, w->pst[c->pnlev - 1], w->cb_null ? 1 : 0, w->pcinv);
}
}  // namespace

void uwg_solver_free(uwg_ctx* c) {
    if (!c->ws.empty()) {
        Work* w = (Work*)c->ws[0];
        if (w->g_v64) cudaGraphExecDestroy(w->g_v64);
        if (w->g_v32) cudaGraphExecDestroy(w->g_v32);
        if (w->g_pv) cudaGraphExecDestroy(w->g_pv);
        if (w->g_lcg) cudaGraphExecDestroy(w->g_lcg);
        if (w->lcg_h) cudaFreeHost(w->lcg_h);
        if (w->gstream) cudaStreamDestroy(w->gstream);
    }
    for (size_t i = 1; i < c->ws.size(); i++) cudaFree(c->ws[i]);
    if (!c->ws.empty()) delete (Work*)c->ws[0];
    c->ws.clear();
}

// Lanczos-free eigenvalue bound: power iteration on D^-1 K with the FP32
// operator (the Chebyshev interval [0.1, 1.2] lambda needs two digits; the FP64
// apply costs 25x more on this GPU's FP64 pipe).
int uwg_solver_estimate(uwg_ctx* c, int l) {
    uwg_level& L = c->lev[l];
    int rc = work_init(c, 30);
    if (rc) return rc;
    Work* w = work_of(c);
    LevelVecs<float>& v = w->v32[l];
    cudaStream_t s = c->stream;
    int64_t n = L.n_dof;
    // deterministic start vector: 1 + small variation, BC dofs zero
    k_power_start<float><<<(unsigned)((n + 255) / 256), 256, 0, s>>>(n, 1.0, 0.37, 0.731, 0.0, v.x);
    vk_mask<float>(s, n, L.bc, v.x);
    double lam = 0.0;
    for (int it = 0; it < 30; it++) {
        if ((rc = uwg_ops_applyK<float>(c, l, v.x, v.t))) return rc;
        vk_mask<float>(s, n, L.bc, v.t);
        vk_pointwise_div<float>(s, n, v.t, L.diag32, v.d);
        double d2[2];
        const float* a[2] = {v.d, v.x};
        const float* b[2] = {v.d, v.x};
        if ((rc = dots<float>(c, n, 2, a, b, d2))) return rc;
        if (d2[1] <= 0.0) break;
        lam = std::sqrt(d2[0] / d2[1]);
        vk_copy<float>(s, n, v.d, v.x);
        vk_scale<float>(s, n, (float)(1.0 / std::sqrt(d2[0])), v.x);
    }
    L.lmax64 = L.lmax32 = lam > 0.0 ? lam : 1.0;
    return UWG_OK;
}

int uwg_solver_setup(uwg_ctx* c) {
    int rc = work_init(c, 50);
    if (rc) return rc;
    for (int l = 0; l < c->nlev; l++) {
        // (level 1 of a Q2 context is assembled from the particles, not coarsened)
        if (l > 0 && c->lev[l - 1].order == 1 && (rc = uwg_ops_coarsen(c, l - 1))) return rc;
        if ((rc = uwg_ops_level_setup(c, l))) return rc;
        if (l < c->nlev - 1 && (rc = uwg_solver_estimate(c, l))) return rc;
    }
    if ((rc = uwg_ops_dense_coarse(c, c->nlev - 1))) return rc;
    // null-space vectors, and whether the checkerboard is a null mode of G (the
    // BFBt pressure multigrid then needs a second rank-one term on its coarsest level)
    {
        Work* w = work_of(c);
        if ((rc = ns_fill(c))) return rc;
        double gn = 1.0;
        if ((rc = g_norm_inf(c, &gn))) return rc;
        vk_copy<double>(c->stream, c->n_pdof, w->ns_t, w->ns_tmp);
        vk_axpy<double>(c->stream, c->n_pdof, -1.0, w->ns_v, w->ns_tmp);
        bool cb = false, cn = false;
        if (c->porder == 0 && (rc = ns_test(c, w->ns_tmp, gn, &cb))) return rc;
        if ((rc = ns_test(c, w->ns_one, gn, &cn))) return rc;
        w->cb_null = cb;
        w->const_null = cn;
    }
    if (c->porder == 0 && (rc = bfbt_setup(c))) return rc;
    return capture_cycles(c, work_of(c)->g_deg > 0 ? work_of(c)->g_deg : 3);
}

extern "C" void uwg_solve_opts_default(uwg_solve_opts* o) {
    if (!o) return;
    o->mixed = 0;
    o->rtol = 1e-8;
    o->inner_rtol = 1e-10;
    o->outer_rtol = 1e-9;
    o->max_inner = 500;
    o->max_outer = 500;
    o->mg_levels = 0;
    o->smooth_steps = 3;
    o->restart = 120;
    o->relax_inner = 1;
    o->schur_pc_smooth = 2;
    o->zero_guess = 1;
    o->schur_pc = 1;
    o->schur_pc_rtol = 3e-2;
    o->p_dir = nullptr;
    o->null_space = 0;
    o->schur_pc_its = 0;
    o->coarse_agg = 0;
    o->coarse_rtol = 1e-2;
}

namespace {

// q = (C - G^T A^-1 G) p  (one inner velocity solve)
int schur_apply(uwg_ctx* c, const SolveCfg& cfg, const double* p, double* q, int* its, int* refine) {
    Work* w = work_of(c);
    int rc;
    if ((rc = uwg_ops_applyG(c, p, w->u_tmp))) return rc;
    int it = 0;
    rc = velocity_solve(c, cfg, w->u_tmp, w->u_tmp2, true, &it, refine);
    *its += it;
    if (rc) return rc;
    if ((rc = uwg_ops_applyGt(c, w->u_tmp2, q))) return rc;
    if ((rc = uwg_ops_apply_C(c, p, w->p_tmp2))) return rc;
    vk_axpby<double>(c->stream, c->n_pdof, 1.0, w->p_tmp2, -1.0, q);
    return UWG_OK;
}

// Right-preconditioned flexible GMRES on the Schur complement, M^-1 = -S^^-1.
int fgmres(uwg_ctx* c, const SolveCfg& cfg, const double* rhs, double* p, double rtol, double atol, int maxit,
           int m, int* its, int* inner_its, int* refine, bool use_p0, const double* z0) {
    Work* w = work_of(c);
    cudaStream_t s = c->stream;
    int64_t n = c->n_pdof;
    int rc;
    double bn;
    const double* ab[1] = {rhs};
    if ((rc = dots<double>(c, n, 1, ab, ab, &bn))) return rc;
    bn = std::sqrt(bn);
    *its = 0;
    if (!use_p0) vk_zero<double>(s, n, p);
    if (bn == 0.0 && !use_p0) return UWG_OK;
    double tol = rtol * bn;
    if (atol > 0.0 && atol < tol) tol = atol;
    std::vector<double> H((m + 1) * m), cs(m), sn(m), g(m + 1), y(m);
    int total = 0;
    // r0 = rhs - S p0 (p0 = 0 unless an initial guess is given)
    vk_copy<double>(s, n, rhs, w->V[0]);
    double beta = bn;
    if (use_p0) {
        if ((rc = schur_apply(c, cfg, p, w->p_tmp, inner_its, refine))) return rc;
        vk_axpy<double>(s, n, -1.0, w->p_tmp, w->V[0]);
        const double* a0[1] = {w->V[0]};
        if ((rc = dots<double>(c, n, 1, a0, a0, &beta))) return rc;
        beta = std::sqrt(beta);
        if (beta <= tol) return UWG_OK;
    }
    while (true) {
        vk_scale<double>(s, n, 1.0 / beta, w->V[0]);
        std::fill(g.begin(), g.end(), 0.0);
        g[0] = beta;
        int j = 0;
        bool done = false;
        for (; j < m && total < maxit; j++) {
            // Z_j = M^-1 V_j: -S^^-1 (the reference's Uzawa term) or scaled BFBt
            double tp0 = now();
            if (z0 && total == 0) {
                // a given first direction (the learned correction) in place of M^-1 V_0
                vk_copy<double>(s, n, z0, w->Z[j]);
            } else if (cfg.schur_pc == 1) {
                if ((rc = bfbt(c, w->V[j], w->Z[j], cfg.schur_pc_rtol, cfg.schur_pc_its))) return rc;
                if (cfg.cc_agg > 0) {
                    // deflation step z = y + Q (r - A y) (uwg_coarse.cu); V[j+1] holds A y until
                    // the iteration's own Schur apply overwrites it
                    SolveCfg cl = cfg;
                    cl.inner_rtol = cfg.cc_rtol;
                    cl.relax = false;
                    if ((rc = schur_apply(c, cl, w->Z[j], w->V[j + 1], inner_its, refine))) return rc;
                    if ((rc = uwg_cc_apply(c, cfg.cc_agg, w->cc_sinv, w->cc_tc, w->cc_zc, w->V[j], w->V[j + 1],
                                           w->Z[j])))
                        return rc;
                    if (w->const_null && (rc = ns_project(c, w->ns_one, w->Z[j]))) return rc;
                }
                double zn;
                const double* az[1] = {w->Z[j]};
                if ((rc = dots<double>(c, n, 1, az, az, &zn))) return rc;
                if (!std::isfinite(zn))
                    return uwg_set_error(c, UWG_ERR_NAN, "non-finite value from the BFBt Schur preconditioner");
                w->t_pc += now() - tp0;
            } else {
                if ((rc = uwg_ops_schur_pc(c, w->V[j], w->Z[j]))) return rc;
                vk_scale<double>(s, n, -1.0, w->Z[j]);
            }
            double ts0 = now();
            // Inexact Krylov (Simoncini & Szyld, SISC 2003): the Schur apply may be
            // less accurate as the residual |g[j]| falls; the true residual is
            // checked with the strict tolerance before returning.
            SolveCfg cj = cfg;
            if (cfg.relax && g[j] != 0.0)
                cj.inner_rtol = std::min(1e-4, std::max(cfg.inner_rtol, cfg.inner_rtol * bn / std::fabs(g[j])));
            if ((rc = schur_apply(c, cj, w->Z[j], w->V[j + 1], inner_its, refine))) return rc;
            w->t_schur += now() - ts0;
            total++;
            // classical Gram-Schmidt, two passes
            std::vector<double> hcol(j + 1, 0.0);
            for (int pass = 0; pass < 2; pass++) {
                for (int i0 = 0; i0 <= j; i0 += 64) {
                    int k = std::min(64, j + 1 - i0);
                    vk_mdot(s, n, k, (const double* const*)w->V.data() + i0, w->V[j + 1], w->coef + i0);
                }
                std::vector<double> hh(j + 1);
                UWG_CUDA(c, cudaMemcpyAsync(hh.data(), w->coef, sizeof(double) * (j + 1), cudaMemcpyDeviceToHost, s));
                UWG_CUDA(c, cudaStreamSynchronize(s));
                for (int i = 0; i <= j; i++) { hcol[i] += hh[i]; hh[i] = -hh[i]; }
                UWG_CUDA(c, cudaMemcpyAsync(w->coef + 256, hh.data(), sizeof(double) * (j + 1), cudaMemcpyHostToDevice, s));
                for (int i0 = 0; i0 <= j; i0 += 64) {
                    int k = std::min(64, j + 1 - i0);
                    vk_maxpy(s, n, k, w->coef + 256 + i0, (const double* const*)w->V.data() + i0, w->V[j + 1]);
                }
            }
            double hn;
            const double* av[1] = {w->V[j + 1]};
            if ((rc = dots<double>(c, n, 1, av, av, &hn))) return rc;
            hn = std::sqrt(hn);
            if (!std::isfinite(hn)) return uwg_set_error(c, UWG_ERR_NAN, "non-finite value in the pressure solve");
            for (int i = 0; i <= j; i++) H[i * m + j] = hcol[i];
            H[(j + 1) * m + j] = hn;
            // apply previous rotations
            for (int i = 0; i < j; i++) {
                double t = cs[i] * H[i * m + j] + sn[i] * H[(i + 1) * m + j];
                H[(i + 1) * m + j] = -sn[i] * H[i * m + j] + cs[i] * H[(i + 1) * m + j];
                H[i * m + j] = t;
            }
            double a = H[j * m + j], b = H[(j + 1) * m + j];
            double r = std::hypot(a, b);
            cs[j] = r == 0.0 ? 1.0 : a / r;
            sn[j] = r == 0.0 ? 0.0 : b / r;
            H[j * m + j] = r;
            H[(j + 1) * m + j] = 0.0;
            g[j + 1] = -sn[j] * g[j];
            g[j] = cs[j] * g[j];
            if (hn > 0.0) vk_scale<double>(s, n, 1.0 / hn, w->V[j + 1]);
            if (std::fabs(g[j + 1]) <= tol || hn == 0.0) { j++; done = true; break; }
        }
        // y = H^-1 g, p += Z y (a zero pivot -- a direction S maps to nothing -- is dropped)
        for (int i = j - 1; i >= 0; i--) {
            double t = g[i];
            for (int k = i + 1; k < j; k++) t -= H[i * m + k] * y[k];
            y[i] = H[i * m + i] != 0.0 ? t / H[i * m + i] : 0.0;
            if (!std::isfinite(y[i])) y[i] = 0.0;
        }
        UWG_CUDA(c, cudaMemcpyAsync(w->coef, y.data(), sizeof(double) * j, cudaMemcpyHostToDevice, s));
        for (int i0 = 0; i0 < j; i0 += 64)
            vk_maxpy(s, n, std::min(64, j - i0), w->coef + i0, (const double* const*)w->Z.data() + i0, p);
        *its = total;
        if (done && !cfg.relax) return UWG_OK;
        if (!done && total >= maxit)
            return uwg_set_error(c, UWG_ERR_NOT_CONVERGED, "pressure solve reached its iteration cap");
        // restart (or, after relaxed applies, confirmation): r = rhs - S p, strict tolerance
        if ((rc = schur_apply(c, cfg, p, w->p_tmp, inner_its, refine))) return rc;
        vk_copy<double>(s, n, rhs, w->V[0]);
        vk_axpy<double>(s, n, -1.0, w->p_tmp, w->V[0]);
        const double* a0[1] = {w->V[0]};
        if ((rc = dots<double>(c, n, 1, a0, a0, &beta))) return rc;
        beta = std::sqrt(beta);
        if (beta <= tol) return UWG_OK;
        if (total >= maxit) return uwg_set_error(c, UWG_ERR_NOT_CONVERGED, "pressure solve reached its iteration cap");
    }
}

}  // namespace

// ||f - Ku - Gp|| and ||h - G^T u - C p|| over free dofs, plus ||f||, ||h||.
int uwg_solver_residuals(uwg_ctx* c, const double* u, const double* p, double* out4) {
    int rc = work_init(c, 30);
    if (rc) return rc;
    Work* w = work_of(c);
    cudaStream_t s = c->stream;
    int64_t nv = c->n_vdof, np = c->n_pdof;
    // momentum: r = f - K u - G p on free dofs (operator includes identity BC rows; mask them)
    if ((rc = uwg_ops_applyK<double>(c, 0, u, w->u_tmp))) return rc;
    if ((rc = uwg_ops_applyG(c, p, w->u_tmp2))) return rc;
    vk_copy<double>(s, nv, c->f, w->ref_r);
    vk_axpy<double>(s, nv, -1.0, w->u_tmp, w->ref_r);
    vk_axpy<double>(s, nv, -1.0, w->u_tmp2, w->ref_r);
    vk_mask<double>(s, nv, c->bc, w->ref_r);
    vk_copy<double>(s, nv, c->f, w->ref_d);
    vk_mask<double>(s, nv, c->bc, w->ref_d);
    // continuity: q = h - G^T u - C p
    if ((rc = uwg_ops_applyGt(c, u, w->p_tmp))) return rc;
    if ((rc = uwg_ops_apply_C(c, p, w->p_tmp2))) return rc;
    vk_axpby<double>(s, np, 1.0, c->h, -1.0, w->p_tmp);
    vk_axpy<double>(s, np, -1.0, w->p_tmp2, w->p_tmp);
    double d[4];
    const double* a2[2] = {w->ref_r, w->ref_d};
    if ((rc = dots<double>(c, nv, 2, a2, a2, d))) return rc;
    const double* a3[2] = {w->p_tmp, c->h};
    if ((rc = dots<double>(c, np, 2, a3, a3, d + 2))) return rc;
    out4[0] = std::sqrt(d[0]);
    out4[1] = std::sqrt(d[2]);
    out4[2] = std::sqrt(d[1]);
    out4[3] = std::sqrt(d[3]);
    return UWG_OK;
}

extern "C" int uwg_stokes_solve(uwg_ctx* c, const uwg_solve_opts* o, double* u, double* p, uwg_solve_stats* st) {
    if (!c || !u || !p) return uwg_set_error(c, UWG_ERR_ARG, "uwg_stokes_solve: bad argument");
    if (!c->assembled) return uwg_set_error(c, UWG_ERR_STATE, "uwg_stokes_solve before uwg_assemble");
    uwg_solve_opts def;
    uwg_solve_opts_default(&def);
    if (!o) o = &def;
    uwg_solve_stats S;
    memset(&S, 0, sizeof(S));
    double t0 = now();
    if (o->restart < 2 || o->restart > 240) return uwg_set_error(c, UWG_ERR_ARG, "restart must be in [2, 240]");
    int rc = work_init(c, o->restart);
    if (rc) return rc;
    Work* w = work_of(c);
    cudaStream_t s = c->stream;
    if (o->schur_pc_smooth < 1 || o->schur_pc_smooth > 16)
        return uwg_set_error(c, UWG_ERR_ARG, "schur_pc_smooth must be in [1, 16]");
    if (o->schur_pc == 1 && c->porder != 0)
        return uwg_set_error(c, UWG_ERR_ARG, "scaled BFBt is implemented for Q1/dQ0; use schur_pc = 0 with Q2/dPc1");
    w->pdeg = o->schur_pc_smooth;
    if (c->porder == 0 && w->pdeg != w->g_pdeg &&
        (rc = capture(c, &w->g_pv, [&]() { return pvcycle(c, 0, w->pcg_r, w->pcg_z); })) == UWG_OK &&
        (rc = capture_lcg(c)) == UWG_OK)
        w->g_pdeg = w->pdeg;
    if (rc) return rc;
    // velocity V-cycle graphs for this smoother degree
    if (std::max(1, o->smooth_steps) != w->g_deg && (rc = capture_cycles(c, std::max(1, o->smooth_steps))))
        return rc;
    int64_t nv = c->n_vdof, np = c->n_pdof;
    // Scaled BFBt approximates (G^T K^-1 G)^-1 only: with a compressible block C the
    // Schur complement C - G^T K^-1 G is preconditioned by the Uzawa term S^ (which holds -C).
    const int schur_pc = (o->schur_pc == 1 && c->compressible) ? 0 : o->schur_pc;
    SolveCfg cfg{o->mixed != 0, o->inner_rtol, o->max_inner, std::max(1, o->smooth_steps), schur_pc,
                 o->schur_pc_rtol > 0.0 ? o->schur_pc_rtol : 1e-2, o->relax_inner != 0, o->schur_pc_its};
    if (o->schur_pc_its < 0 || o->schur_pc_its > 200) return uwg_set_error(c, UWG_ERR_ARG, "schur_pc_its must be in [0, 200]");
    // coarse-level correction: BFBt, incompressible, no checkerboard null mode (its
    // aggregates would not see it); Sc^-1 is rebuilt after each assembly
    if (o->coarse_agg < 0) return uwg_set_error(c, UWG_ERR_ARG, "coarse_agg must be >= 0");
    if (o->coarse_agg > 0 && schur_pc == 1 && !c->compressible && !w->cb_null) {
        int npc = 0, lv = 0;
        if (uwg_cc_dims(c, o->coarse_agg, &npc, &lv) == 0 && npc > w->cc_cap && npc <= 1024) {
            if (!(w->cc_sinv = dalloc<double>(c, (int64_t)npc * npc)) || !(w->cc_tc = dalloc<double>(c, npc)) ||
                !(w->cc_zc = dalloc<double>(c, npc)))
                return uwg_set_error(c, UWG_ERR_CUDA, "coarse correction: out of device memory");
            w->cc_cap = npc;
            w->cc_gen = -1;
        }
        if (w->cc_gen != c->asm_gen || w->cc_agg != o->coarse_agg) {
            double tc0 = now();
            if ((rc = uwg_cc_build(c, o->coarse_agg, w->const_null, w->cc_sinv))) return rc;
            w->cc_gen = c->asm_gen;
            w->cc_agg = o->coarse_agg;
            S.coarse_setup_time = now() - tc0;
        }
        cfg.cc_agg = o->coarse_agg;
        cfg.cc_rtol = o->coarse_rtol > 0.0 ? o->coarse_rtol : 1e-2;
        S.coarse_dim = npc;
    }
    // b = f with Dirichlet values in BC rows
    vk_copy<double>(s, nv, c->f, w->bvec);
    {
        // bvec[bc] = bcval[bc]
        vk_mask<double>(s, nv, c->bc, w->bvec);
        // add values: bvec += bcval (bcval is zero on free dofs)
        vk_axpy<double>(s, nv, 1.0, c->bcval, w->bvec);
    }
    double t1 = now();
    S.setup_time = t1 - t0;
    // 1. pre-solve
    int it = 0;
    rc = velocity_solve(c, cfg, w->bvec, w->ftil, true, &it, &S.refinement_steps);
    S.velocity_presolve_its = it;
    S.fhat_reason = rc ? -1 : 1;
    if (rc) return rc;
    // zero BC entries of f~ (the reduced system excludes them)
    vk_mask<double>(s, nv, c->bc, w->ftil);
    double t2 = now();
    S.presolve_time = t2 - t1;
    // null-space vectors requested by the caller that lie in the null space of G
    // (KSPBuildPressure_*_Nullspace_BSSCR + the test of KSPRemovePressureNullspace_BSSCR)
    const double* nsv[2];
    int n_ns = 0;
    double gnorm = 1.0;
    if ((rc = g_norm_inf(c, &gnorm))) return rc;
    if (o->null_space < 0 || o->null_space > 2) return uwg_set_error(c, UWG_ERR_ARG, "null_space must be 0, 1 or 2");
    if (o->null_space) {
        const double* cand[2] = {o->null_space == 1 ? w->ns_one : w->ns_t, o->null_space == 1 ? nullptr : w->ns_v};
        for (int k = 0; k < 2; k++) {
            bool in_ns = false;
            if (cand[k] && (rc = ns_test(c, cand[k], gnorm, &in_ns))) return rc;
            if (in_ns) nsv[n_ns++] = cand[k];
        }
        // The components of h along them make the system inconsistent; they are
        // dropped from h itself, so that the reported residual is the consistent system's.
        for (int k = 0; k < n_ns; k++)
            if ((rc = ns_project(c, nsv[k], c->h))) return rc;
    }
    // 2. h^ = h - G^T f~
    if ((rc = uwg_ops_applyGt(c, w->ftil, w->hhat))) return rc;
    vk_axpby<double>(s, np, 1.0, c->h, -1.0, w->hhat);
    for (int k = 0; k < n_ns; k++)
        if ((rc = ns_project(c, nsv[k], w->hhat))) return rc;
    // 3. pressure solve: S p = h^, S = C - G^T A^-1 G
    w->lsolve_its = 0;
    w->t_pc = w->t_schur = 0.0;
    int outer = 0, inner_its = 0;
    // the full-system target ||[f - Ku - Gp; h - G^T u]|| <= rtol ||[f; h]|| is met once the
    // Schur residual is below it (the back-solve adds inner_rtol-level error)
    double fh2[2];
    {
        vk_copy<double>(s, nv, c->f, w->u_tmp);
        vk_mask<double>(s, nv, c->bc, w->u_tmp);
        const double* a1[1] = {w->u_tmp};
        if ((rc = dots<double>(c, nv, 1, a1, a1, &fh2[0]))) return rc;
        const double* a2[1] = {c->h};
        if ((rc = dots<double>(c, np, 1, a2, a2, &fh2[1]))) return rc;
    }
    double atol = o->rtol > 0.0 ? 0.5 * o->rtol * std::sqrt(fh2[0] + fh2[1]) : 0.0;
    // h^ scaling (auglag-driver-DGTGD.c:410-417): a small ||h^|| / ||G||_inf in
    // (1e-20, 1e-6) is scaled to one for the pressure solve and p scaled back after.
    double hscale = 1.0;
    {
        double hn;
        const double* ah[1] = {w->hhat};
        if ((rc = dots<double>(c, np, 1, ah, ah, &hn))) return rc;
        hn = std::sqrt(hn) / gnorm;
        if (hn < 1e-6 && hn > 1e-20) hscale = 1.0 / hn;
    }
    if (hscale != 1.0) {
        vk_scale<double>(s, np, hscale, w->hhat);
        if (o->zero_guess == 0) vk_scale<double>(s, np, hscale, p);
        atol *= hscale;
    }
    rc = fgmres(c, cfg, w->hhat, p, o->outer_rtol, atol, o->max_outer, std::max(2, o->restart), &outer, &inner_its,
                &S.refinement_steps, o->zero_guess == 0, o->p_dir);
    if (hscale != 1.0) vk_scale<double>(s, np, 1.0 / hscale, p);
    for (int k = 0; !rc && k < n_ns; k++) rc = ns_project(c, nsv[k], p);
    S.pressure_its = outer;
    S.schur_pc_its = w->lsolve_its;
    S.schur_pc_used = schur_pc;
    S.schur_pc_time = w->t_pc;
    S.schur_op_time = w->t_schur;
    S.velocity_pressuresolve_its = inner_its;
    S.outer_reason = rc ? -1 : 1;
    if (rc) {
        S.velocity_total_its = S.velocity_presolve_its + S.velocity_pressuresolve_its;
        S.total_time = now() - t0;
        if (st) *st = S;   // partial statistics of the failed solve
        return rc;
    }
    double t3 = now();
    S.pressure_time = t3 - t2;
    // 4. back-solve: A u = b - G p
    if ((rc = uwg_ops_applyG(c, p, w->u_tmp))) return rc;
    vk_copy<double>(s, nv, w->bvec, w->cg_q);
    vk_axpy<double>(s, nv, -1.0, w->u_tmp, w->cg_q);
    vk_copy<double>(s, nv, w->cg_q, w->u_tmp2);
    rc = velocity_solve(c, cfg, w->u_tmp2, u, o->zero_guess != 0, &it, &S.refinement_steps);
    S.velocity_backsolve_its = it;
    S.backsolve_reason = rc ? -1 : 1;
    if (rc) return rc;
    double t4 = now();
    S.backsolve_time = t4 - t3;
    S.velocity_total_its = S.velocity_presolve_its + S.velocity_pressuresolve_its + S.velocity_backsolve_its;
    double r4[4];
    if ((rc = uwg_solver_residuals(c, u, p, r4))) return rc;
    double num = std::sqrt(r4[0] * r4[0] + r4[1] * r4[1]);
    double den = std::sqrt(r4[2] * r4[2] + r4[3] * r4[3]);
    S.residual = den > 0.0 ? num / den : num;
    S.total_time = now() - t0;
    if (st) *st = S;
    return UWG_OK;
}

extern "C" int uwg_stokes_residuals(uwg_ctx* c, const double* u, const double* p, double* res_h) {
    if (!c || !u || !p || !res_h) return uwg_set_error(c, UWG_ERR_ARG, "uwg_stokes_residuals: bad argument");
    if (!c->assembled) return uwg_set_error(c, UWG_ERR_STATE, "residuals before uwg_assemble");
    double r4[4];
    int rc = uwg_solver_residuals(c, u, p, r4);
    if (rc) return rc;
    res_h[0] = r4[0];
    res_h[1] = r4[1];
    return UWG_OK;
}
