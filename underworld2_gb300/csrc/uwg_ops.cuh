// Operator kernels of the Stokes system on regular Q1/dQ0 meshes (declarations).
#pragma once
#include "uwg_internal.cuh"

// Geometry of one level passed by value to kernels.
struct uwg_lgeom {
    int dim, order;
    int res[3];
    int nx[3];
    const double* ax[3];
    int64_t n_el, n_nodes;
};

uwg_lgeom uwg_level_geom(const uwg_ctx* c, int l);
int64_t uwg_ops_ktiles(const int* res);   // tiles of the 3D Q1 tiled apply

// Assembly from the PIC swarm (finest level): W, f, Mp.
int uwg_ops_assemble(uwg_ctx* c, const int32_t* off, const int32_t* list, const double* ip_xi,
                     const double* ip_w, const double* eta_p, const double* body_p, const double* lambda_p);
// Per-level derived data: diag (and Shat on level 0), W32 copy, coarsening.
int uwg_ops_level_setup(uwg_ctx* c, int l);
int uwg_ops_coarsen(uwg_ctx* c, int l);          // W of level l+1 from level l
int uwg_ops_bc_coarsen(uwg_ctx* c, int l);       // BC mask of level l+1 from level l
int uwg_ops_dense_coarse(uwg_ctx* c, int l);     // dense inverse of level l
int uwg_ops_dense_matrix(uwg_ctx* c, int l, double* A);   // dense operator of level l (Dirichlet rows: identity)
// Coarse-level correction of the Schur FGMRES (uwg_coarse.cu): aggregates per
// pressure multigrid / velocity level (0, or -1 not 2D Q1/dQ0, -2 bad agg, -3 no level),
// Sc^-1 into sinv [npc^2], and z -= P Sc^-1 P^T (r - s).
int uwg_cc_dims(const uwg_ctx* c, int agg, int* npc, int* lv);
int uwg_cc_build(uwg_ctx* c, int agg, bool const_null, double* sinv);
int uwg_cc_apply(uwg_ctx* c, int agg, const double* sinv, double* tc, double* zc, const double* r, const double* s,
                 double* z);

template <typename T> int uwg_ops_applyK(uwg_ctx* c, int l, const T* x, T* y);
template <typename T> int uwg_ops_prolong_add(uwg_ctx* c, int lc, const T* xc, T* xf);   // xf += P xc
template <typename T> int uwg_ops_restrict(uwg_ctx* c, int lc, const T* rf, T* rc);       // rc = R rf
template <typename T> int uwg_ops_dense_solve(uwg_ctx* c, int l, const T* b, T* x);
int uwg_ops_applyG(uwg_ctx* c, const double* p, double* y);      // y = G p (BC rows zero)
int uwg_ops_applyGt(uwg_ctx* c, const double* u, double* q);     // q = G^T u (BC dofs ignored)
int uwg_ops_applyGt_mode(uwg_ctx* c, const double* u, double* q, int only_bc);
int uwg_ops_applyK_lift(uwg_ctx* c, const double* x, double* y); // y = P K x, x unmasked
int uwg_solver_setup(uwg_ctx* c);
void uwg_solver_free(uwg_ctx* c);
int uwg_solver_residuals(uwg_ctx* c, const double* u, const double* p, double* out4);
int uwg_ops_schur_pc(uwg_ctx* c, const double* r, double* z);    // z = Shat^-1 r
int uwg_ops_applyL(uwg_ctx* c, int l, const double* p, double* q, double* vtmp);  // q = G^T D^-1 G p
int uwg_ops_Ldiag(uwg_ctx* c, int l, double* out);
int uwg_ops_cell_restrict(uwg_ctx* c, int lc, const double* rf, double* rc);
int uwg_ops_G32(uwg_ctx* c, int l, const float* Dinv, const float* p, float* v);
int uwg_ops_Gt32(uwg_ctx* c, int l, const float* v, float* q);
int uwg_ops_applyL32(uwg_ctx* c, int l, const float* Dinv, const float* p, float* q, float* vtmp);
int uwg_ops_Ldiag32(uwg_ctx* c, int l, const float* Dinv, float* out);
int uwg_ops_winv(uwg_ctx* c, int l, float* out);
int uwg_ops_cell_restrict32(uwg_ctx* c, int lc, const float* rf, float* rc);
int uwg_ops_cell_prolong_add32(uwg_ctx* c, int lc, const float* xc, float* xf);
int uwg_ops_cell_prolong_add(uwg_ctx* c, int lc, const double* xc, double* xf);
int uwg_ops_apply_C(uwg_ctx* c, const double* p, double* q);     // q = Mp p (compressibility)
int uwg_ops_element_matrices(uwg_ctx* c, int64_t el, double* Ke, double* fe, double* Ge, double* Se);

// Q2/dPc1 (uwg_q2.cu): level 0 operators of Q2 contexts
int uwg_q2_init(uwg_ctx* c);
int uwg_q2_assemble(uwg_ctx* c, const int32_t* off, const int32_t* list, const double* ip_xi, const double* ip_w,
                    const double* eta_p, const double* body_p);
template <typename T> int uwg_q2_applyK(uwg_ctx* c, const T* x, T* y, bool mask_in);
int uwg_q2_diag(uwg_ctx* c, double* sinv);
int uwg_q2_applyG(uwg_ctx* c, const double* p, double* y);
int uwg_q2_applyGt(uwg_ctx* c, const double* u, double* q, int only_bc);
int uwg_q2_schur_pc(uwg_ctx* c, const double* r, double* z);
int uwg_q2_element_matrices(uwg_ctx* c, int64_t el, double* Ke, double* Ge, double* Se);
// 3D Q2/dPc1 (uwg_q2_3d.cu), dispatched from the uwg_q2_* entry points
int uwg_q2_3d_init(uwg_ctx* c);
int uwg_q2_3d_assemble(uwg_ctx* c, const int32_t* off, const int32_t* list, const double* ip_xi, const double* ip_w,
                       const double* eta_p, const double* body_p);
template <typename T> int uwg_q2_3d_applyK(uwg_ctx* c, const T* x, T* y, bool mask_in);
int uwg_q2_3d_applyK_df(uwg_ctx* c, const double* x, double* y);
// The velocity operator for refinement residuals: double-float on 3D Q2 meshes
// with stored element matrices, else the FP64 apply.
int uwg_ops_applyK_refine(uwg_ctx* c, const double* x, double* y);
int uwg_q2_3d_diag(uwg_ctx* c, double* sinv);
int uwg_q2_3d_applyG(uwg_ctx* c, const double* p, double* y);
int uwg_q2_3d_applyGt(uwg_ctx* c, const double* u, double* q, int only_bc);
int uwg_q2_3d_schur_pc(uwg_ctx* c, const double* r, double* z);
int uwg_q2_3d_element_matrices(uwg_ctx* c, int64_t el, double* Ke, double* Ge, double* Se);

int uwg_ops_dense_invert(uwg_ctx* c, int64_t n, double* A, double* B);   // B = A^-1 (A destroyed)
int uwg_ops_dense_invert_grid(uwg_ctx* c, int64_t n, double* A, double* B);   // the same, grid-wide steps
int uwg_ops_to_f32(uwg_ctx* c, int64_t n, const double* a, float* b);
int uwg_ops_dense_mv32(uwg_ctx* c, int64_t n, const float* Ainv, const float* b, float* x);

// Pressure-Laplacian multigrid of the weighted BFBt preconditioner (uwg_pmg.cu).
// Level 0 has one unknown per cell, coarser levels two (smooth, checkerboard).
int uwg_pmg_ncomp(int l);
int64_t uwg_pmg_stencil_size(const uwg_ctx* c, int l);
// level 0: stencil of G^T W G from W0; level l > 0: Galerkin product of st_fine
int uwg_pmg_stencil(uwg_ctx* c, int l, const float* W0, const float* st_fine, float* st);
int uwg_pmg_apply(uwg_ctx* c, int l, const float* st, const float* x, float* y);
int uwg_pmg_apply0_mf(uwg_ctx* c, const float* W0, const float* x, float* y);   // level 0, 3D, no stencil
int uwg_pmg_diag(uwg_ctx* c, int l, const float* st, float* d);
int uwg_pmg_restrict(uwg_ctx* c, int lc, const float* rf, float* rc);
int uwg_pmg_prolong_add(uwg_ctx* c, int lc, const float* xc, float* xf);
int uwg_pmg_dense_inverse(uwg_ctx* c, int l, const float* st, int fix_checkerboard, float* inv32);

// Vector kernels ---------------------------------------------------------------
template <typename T> void vk_copy(cudaStream_t s, int64_t n, const T* x, T* y);
template <typename A, typename B> void vk_convert(cudaStream_t s, int64_t n, const A* x, B* y);
template <typename T> void vk_axpy(cudaStream_t s, int64_t n, T a, const T* x, T* y);          // y += a x
template <typename T> void vk_axpby(cudaStream_t s, int64_t n, T a, const T* x, T b, T* y);    // y = a x + b y
template <typename T> void vk_scale(cudaStream_t s, int64_t n, T a, T* y);
template <typename T> void vk_zero(cudaStream_t s, int64_t n, T* y);
template <typename T> void vk_mask(cudaStream_t s, int64_t n, const uint8_t* bc, T* y);       // y[bc] = 0
template <typename T> void vk_cheb(cudaStream_t s, int64_t n, const T* b, const T* t, const T* diag, T a, T c, T* d,
                                   T* x, int first, int x_zero);
template <typename T> void vk_pointwise_div(cudaStream_t s, int64_t n, const T* x, const T* d, T* y);
// Sums of products into dst[k] (double), k < 4: dots of (a_k, b_k) pairs.
template <typename T> void vk_dots(cudaStream_t s, int64_t n, int k, const T* const* a, const T* const* b,
                                   double* dst);
void vk_mdot(cudaStream_t s, int64_t n, int k, const double* const* V, const double* w, double* dst);
void vk_pointwise_mul_mask(cudaStream_t s, int64_t n, const float* w, float* y);
void vk_maxpy(cudaStream_t s, int64_t n, int k, const double* coef_dev, const double* const* V, double* y);
