/*
 * uwg.h -- C ABI of libuwg, the GB300 (sm_103a) particle-in-cell Stokes path.
 *
 * Conventions
 *   - Every array argument is a DEVICE pointer unless its name ends in _h.
 *   - The caller owns particle arrays; a context owns the mesh geometry, the
 *     assembled operators and the solver workspaces.
 *   - Every call is ordered on the context's stream (uwg_set_stream) and
 *     returns UWG_OK (0) or a negative UWG_ERR_* code; uwg_last_error()
 *     gives the message.  Calls that return values to the host
 *     (statistics, counts, dt) synchronise the stream before returning.
 *   - No exception or device trap crosses this boundary.
 *
 * Each entry point names the reference native call it replaces; the Python
 * layer in underworld2_gb300/ calls them where underworld2's Python layer
 * calls those functions through SWIG.  Citations:
 *   L/ = src/underworld/libUnderworld/,  P/ = src/underworld/
 */
#ifndef UWG_H
#define UWG_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define UWG_OK 0
#define UWG_ERR_ARG (-1)            /* invalid argument */
#define UWG_ERR_CUDA (-2)           /* CUDA runtime failure */
#define UWG_ERR_STATE (-3)          /* call out of order (e.g. solve before assemble) */
#define UWG_ERR_EMPTY_CELL (-4)     /* an element holds no particle (DVC needs >= 1) */
#define UWG_ERR_CELL_FULL (-5)      /* more particles in one element than the kernels hold */
#define UWG_ERR_NOT_CONVERGED (-6)  /* a Krylov solve hit its iteration cap */
#define UWG_ERR_NAN (-7)            /* non-finite value met in a solve */
#define UWG_ERR_PARTICLE_LOST (-8)  /* particles left the domain */

typedef struct uwg_ctx uwg_ctx;

/* Mesh description: regular Cartesian box, Q1 (order 1) or Q2 (order 2)
 * velocity elements, dQ0 (porder 0) or dPc1 (porder 1) pressure.
 * Replaces FeMesh_Cartesian construction (P/mesh/_mesh.py:1105-1160) over
 * CartesianGenerator / C2Generator (L/StgDomain/Mesh/src/CartesianGenerator.c,
 * L/StgFEM/Discretisation/src/C2Generator.c). */
typedef struct {
    int dim;
    int order;
    int porder;
    int res[3];
    double minc[3];
    double maxc[3];
} uwg_mesh_desc;

int uwg_ctx_create(const uwg_mesh_desc* desc, uwg_ctx** out);
void uwg_ctx_destroy(uwg_ctx* ctx);
const char* uwg_last_error(const uwg_ctx* ctx);
int uwg_set_stream(uwg_ctx* ctx, void* cuda_stream);
int uwg_sync(uwg_ctx* ctx);
/* sizes: n_el, n_nodes (velocity), n_vdof, n_pdof, nen, npn */
int uwg_mesh_sizes(const uwg_ctx* ctx, int64_t* sizes_h);
/* node coordinates per axis, copied to host arrays of length res*order+1 */
int uwg_mesh_axis(const uwg_ctx* ctx, int axis, double* coords_h);

/* ---- Function-graph evaluation at integration points --------------------------
 * One op of a register program: r[dst] = f(r[a], r[b], imm) (opcodes in
 * csrc/uwg_fn.cu; function.py compiles the graph).  An input is an array of
 * `count` components per row, of dtype 0 f64, 1 f32, 2 i32, 3 i8, 4 i16, 5 i64,
 * indexed by the point's particle id (by_particle = 1) or by the point index. */
typedef struct {
    int32_t op, dst, a, b;
    double imm;
} uwg_fn_op;
typedef struct {
    const void* ptr;
    int32_t dtype, count, by_particle, pad;
} uwg_fn_input;

/* Evaluates the program at n points (pid[n]: particle of each point, or NULL)
 * into out[n][nout], or into out[pid[i]][nout] with out_by_particle; *flags_h
 * collects the program's error checks (bit k set by a failing check with
 * code k).  Replaces the per-point virtual-call
 * evaluation of the function graph behind the assembly terms
 * (L/Underworld/Function/src/SwarmVariableFn.cpp:30-110, Map.cpp,
 * Conditional.cpp, MathUnary.cpp, Arithmetic.cpp). */
int uwg_fn_eval(uwg_ctx* ctx, int nops, const uwg_fn_op* ops_h, int ninputs, const uwg_fn_input* inputs_h,
                int64_t n, const int32_t* pid, int nout, int out_by_particle, double* out, int32_t* flags_h);

/* Seeded per-cell uniform-random particle layout: cells in order, particles
 * in order, dims in order, one Park-Miller stream seeded with seed^123459876.
 * Writes x[n_el*ppc][dim], owner[n_el*ppc] and the cell tables
 * (cell_offsets[n_el+1], cell_list[n_el*ppc]).  *rng_state_h is the stream
 * state before the first draw and is advanced past the last one.
 * Replaces ParticleLayout_InitialiseParticles for PerCellRandomLayout
 * (L/StgFEM/Utils/src/MeshParticleLayout.c:194-230,
 *  L/StgDomain/Swarm/src/Random.c:23-53, P/swarm/layouts.py:186-231). */
int uwg_layout_random(uwg_ctx* ctx, int ppc, int64_t* rng_state_h, double* x, int32_t* owner,
                      int32_t* cell_offsets, int32_t* cell_list);

/* Element that owns each particle (n_el when outside the mesh), no table
 * edits.  Replaces CellLayout_CellOf / _ElementCellLayout_CellOf
 * (L/StgDomain/Swarm/src/ElementCellLayout.c:291-320) over
 * Mesh_RegularAlgorithms_SearchElements (L/StgDomain/Mesh/src/Mesh_RegularAlgorithms.c:174-205). */
int uwg_locate(uwg_ctx* ctx, int64_t np, const double* x, int32_t* owner);

/* Material particle of each Gauss integration point, for swarm-variable functions
 * evaluated on a Gauss integration swarm.  Replaces GeneralSwarm_IntegrationPointMap
 * (L/PICellerator/MaterialPoints/src/GeneralSwarm.cpp:319-431, called from
 * SwarmVariableFn, L/Underworld/Function/src/SwarmVariableFn.cpp:73-101): the
 * point's global position by FeMesh_CoordLocalToGlobal, then the first particle of
 * its element's cell list at the least squared distance.
 *   xi_q          [nq*dim] local coordinates of the element's points (device)
 *   cell_offsets, cell_list, x   the swarm's cell tables and coordinates (device)
 *   pid           [n_el*nq] out: particle index per point, element-major; -1 where
 *                 the element holds no particle (the reference raises there) */
int uwg_gauss_nearest(uwg_ctx* ctx, int nq, const double* xi_q, const int32_t* cell_offsets,
                      const int32_t* cell_list, const double* x, int32_t* pid);

/* Owner update with the reference's cell-table semantics: particles are
 * visited in index order, a leaver is removed from its old cell by
 * swap-with-last, an arrival is appended.  cell_offsets/cell_list are
 * rewritten in place.  *n_lost_h = particles now outside the mesh (their
 * owner is n_el).  Replaces Swarm_UpdateAllParticleOwners
 * (L/StgDomain/Swarm/src/SwarmClass.c:947-1015). */
int uwg_update_owners(uwg_ctx* ctx, int64_t np, const double* x, int32_t* owner,
                      int32_t* cell_offsets, int32_t* cell_list, int64_t* n_lost_h);

/* Coincident mapping: the local coordinate of every particle in its element,
 * by the Newton iteration of _ElementType_ConvertGlobalCoordToElLocal.
 * ip_xi is written in cell-table slot order: [cell_offsets[e]+k][dim] is
 * particle cell_list[cell_offsets[e]+k].  Replaces _CoincidentMapper_Map
 * (L/PICellerator/MaterialPoints/src/CoincidentMapper.c:76-125,
 *  L/StgFEM/Discretisation/src/ElementType.c:177-301). */
int uwg_pic_map(uwg_ctx* ctx, int64_t np, const double* x, const int32_t* cell_offsets,
                const int32_t* cell_list, double* ip_xi);

/* Discrete Voronoi cell weights on a res^dim grid per element: ip_xi is
 * replaced by the centroid of each particle's cells, ip_w = cells * cell
 * volume.  Slot order as uwg_pic_map.  Replaces WeightsCalculator_CalculateAll
 * with DVCWeights (L/PICellerator/Weights/src/DVCWeights.c:772-927). */
int uwg_dvc_weights(uwg_ctx* ctx, int res, const int32_t* cell_offsets, double* ip_xi,
                    double* ip_w);

/* DVC weights without any device allocation and without a context.
 * No counterpart in the reference: it exists for callers that cannot allocate
 * device memory when they need the weights -- host frameworks that reserve the
 * GPU's memory in their own pool at start-up and forbid later cudaMalloc calls,
 * and plugin hosts that hand a plugin device buffers but no allocator -- and
 * that therefore cannot create a context (creating one allocates).
 * Same inputs and outputs as uwg_dvc_weights (dim 2 or 3, res 1..16, at most
 * 128 particles per element), on `cuda_stream`; reads the status word back
 * and synchronises the stream before it returns.
 * The boundary-list scratch is a fixed 32 MiB device array inside libuwg that
 * every GPU loading the library holds until exit; the first call on a device
 * looks its address up (cudaGetSymbolAddress) and keeps it, so a device must
 * not be reset (cudaDeviceReset) between calls.  All calls share that array
 * and its status word, which each call clears first: calls that overlap on the
 * GPU (different streams or threads) race and must be serialised by the caller.
 * Returns 0, UWG_ERR_ARG, UWG_ERR_CUDA, UWG_ERR_EMPTY_CELL, UWG_ERR_CELL_FULL or UWG_ERR_STATE
 * (a listed particle's local coordinates lie outside [-1, 1]). */
int uwg_dvc_weights_noalloc(int dim, int res, int64_t n_el, const int32_t* cell_offsets, double* ip_xi,
                            double* ip_w, void* cuda_stream);

/* Dirichlet conditions: bc_mask[n_vdof] (1 = fixed), values[n_vdof].
 * Replaces FeVariable_SetBC + SystemLinearEquations_BC_Setup
 * (P/systems/_stokes.py:194-204, L/StgFEM/SLE/SystemSetup/src/SystemLinearEquations.c:521). */
int uwg_set_bcs(uwg_ctx* ctx, const uint8_t* bc_mask, const double* values);

/* Assembly of the Stokes operators from the PIC integration swarm:
 *  - viscous operator K from the points (ip_xi, ip_w) with per-particle
 *    viscosity eta_p (stored as exact equivalent-quadrature weights per element);
 *  - f from the body force body_p[np][dim] at the points;
 *  - G from Gauss quadrature (geometry only);
 *  - the Schur preconditioner S_e = G_e^T diag(K_e)^-1 G_e;
 *  - optional compressibility (pressure mass) from lambda_p (may be NULL);
 *  - Dirichlet lifting of f and h.
 * Replaces SystemLinearEquations_MatrixSetup / VectorSetup
 * (L/StgFEM/SLE/SystemSetup/src/StiffnessMatrix.c:552-744, ForceVector.c:231-361)
 * with the terms ConstitutiveMatrixCartesian (L/Underworld/Rheology/src/
 * ConstitutiveMatrixCartesian.cpp:238-429), GradientStiffnessMatrixTerm
 * (L/StgFEM/Assembly/src/GradientStiffnessMatrixTerm.c:129-219),
 * UzawaPreconditionerTerm (L/StgFEM/SLE/ProvidedSystems/StokesFlow/src/
 * UzawaPreconditionerTerm.c:124-207), VectorAssemblyTerm_NA__Fn and
 * MatrixAssemblyTerm_NA__NB__Fn (L/Underworld/Utils/src/). */
int uwg_assemble(uwg_ctx* ctx, int64_t np, const int32_t* cell_offsets, const int32_t* cell_list,
                 const double* ip_xi, const double* ip_w, const double* eta_p,
                 const double* body_p, const double* lambda_p);

/* Adds df[n_vdof] (device) to the assembled velocity right-hand side at free dofs:
 * the traction (NeumannCondition) surface term VectorSurfaceAssemblyTerm_NA__Fn__ni
 * (L/Underworld/Utils/src/VectorSurfaceAssemblyTerm_NA__Fn__ni.cpp:163-236), which the
 * reference adds to the Stokes force vector (P/systems/_stokes.py:291-297).  Call after
 * uwg_assemble, which rebuilds the right-hand side. */
int uwg_add_force(uwg_ctx* ctx, const double* df);

/* Adds the continuity source term to the assembled pressure right-hand side:
 * h_e[b] += sum_q w_q detJ src_q M_b(xi_q) over the PIC points (slot order as
 * uwg_assemble; src_p per particle).  Replaces the VectorAssemblyTerm_NA__Fn on the
 * pressure vector (L/Underworld/Utils/src/VectorAssemblyTerm_NA__Fn.cpp:143-202) that
 * P/systems/_stokes.py:284-288 builds for fn_source.  Call after uwg_assemble. */
int uwg_add_source(uwg_ctx* ctx, const int32_t* cell_offsets, const int32_t* cell_list, const double* ip_xi,
                   const double* ip_w, const double* src_p);

/* Element matrices of one element as assembled (host outputs, for checks):
 * Ke_h[(dim*nen)^2], fe_h[dim*nen], Ge_h[dim*nen*npn], Se_h[npn*npn]. */
int uwg_element_matrices(uwg_ctx* ctx, int64_t el, double* Ke_h, double* fe_h, double* Ge_h,
                         double* Se_h);

typedef struct {
    int mixed;             /* 0: plain FP64 inner solves, 1: FP32 inner solves with FP64 refinement */
    double rtol;           /* target ||[f-Ku-Gp ; h-G^T u]|| / ||[f;h]|| */
    double inner_rtol;     /* relative tolerance of each velocity solve */
    double outer_rtol;     /* relative tolerance of the Schur solve */
    int max_inner;
    int max_outer;
    int mg_levels;         /* 0 = reference rule (halvings + 1) */
    int smooth_steps;      /* Chebyshev degree per smoothing */
    int restart;           /* FGMRES restart length */
    int zero_guess;        /* 1: start from u=p=0, else from the given u, p */
    int schur_pc;          /* 0: assembled Uzawa term S^ (the reference's "uw"), 1: scaled BFBt */
    double schur_pc_rtol;  /* relative tolerance of the pressure-Laplacian solves inside BFBt */
    int relax_inner;       /* 1: loosen the velocity-solve tolerance inside the Schur iteration as its
                              residual falls (inexact Krylov), then confirm with one strict residual */
    int schur_pc_smooth;   /* Chebyshev degree of the pressure-multigrid smoother inside BFBt */
    const double* p_dir;   /* device [n_pdof] or NULL: first search direction of the Schur FGMRES in
                              place of the first preconditioner application (a learned correction;
                              the least-squares step of the iteration chooses its weight) */
    int null_space;        /* pressure null-space removal (KSPRemovePressureNullspace_BSSCR,
                              L/Solvers/KSPSolvers/src/BSSCR/ksp_pressure_nullspace.c:28-183):
                              0 none (the reference's default); 1 the constant
                              (remove_constant_pressure_null_space); 2 the even-cell and odd-cell
                              indicator vectors (-remove_checkerboard_pressure_null_space), which
                              span the constant and the Q1/dQ0 checkerboard.  A vector is removed
                              only if ||G t||/||t|| < 1e-7 ||G||_inf: from h (and h^) before the
                              pressure solve and from p after it. */
    int schur_pc_its;      /* > 0: each pressure-Laplacian solve inside BFBt runs this many CG
                              iterations (rounded up to even) instead of stopping at schur_pc_rtol */
    int coarse_agg;        /* > 0 (2D Q1/dQ0, BFBt, incompressible): coarse-level correction inside
                              the flexible GMRES.  Pressure cells are aggregated in coarse_agg x
                              coarse_agg blocks; the coarse Schur complement Sc = Gc^T Kc^-1 Gc is
                              built from the velocity multigrid level whose elements are
                              coarse_agg / 2 fine cells wide (Galerkin Kc, exact Gc) and inverted
                              densely; each preconditioner application is the deflation step
                              z = y + Q (r - S y), y = BFBt(r), Q = P Sc^-1 P^T (one extra Schur
                              apply at coarse_rtol).  No counterpart in the reference. */
    double coarse_rtol;    /* velocity tolerance of the extra Schur apply (default 1e-2) */
} uwg_solve_opts;

typedef struct {
    int pressure_its;
    int velocity_presolve_its;
    int velocity_pressuresolve_its;
    int velocity_backsolve_its;
    int velocity_total_its;
    int refinement_steps;
    double setup_time, presolve_time, pressure_time, backsolve_time, total_time;
    double residual;       /* final relative residual of the full system, FP64 */
    double vmin, vmax, pmin, pmax;
    int fhat_reason, outer_reason, backsolve_reason; /* >0 converged, <0 not */
    int schur_pc_its;      /* CG iterations of the pressure-Laplacian solves inside BFBt */
    double schur_pc_time;  /* seconds in the Schur preconditioner */
    double schur_op_time;  /* seconds in Schur-operator applications (inner velocity solves) */
    int schur_pc_used;     /* the Schur preconditioner applied: schur_pc, except that a compressible
                              system (pressure block C) is preconditioned by the Uzawa term (0) */
    int coarse_dim;        /* dimension of the coarse space of the correction (0: not used) */
    double coarse_setup_time; /* seconds building Sc^-1 */
} uwg_solve_stats;

void uwg_solve_opts_default(uwg_solve_opts* o);

/* BSSCR Schur-complement solve: f~ = K^-1 f, h^ = h - G^T f~, solve
 * (G^T K^-1 G) p = -h^ with the Schur preconditioner, then K u = f - G p.
 * u[n_vdof] (node-major, dof-minor, Dirichlet dofs carry their values) and
 * p[n_pdof] in/out.  Replaces SystemLinearEquations_ExecuteSolver ->
 * _StokesBlockKSPInterface_Solve -> KSPSolve_BSSCR -> BSSCR_DRIVER_auglag
 * (L/Solvers/KSPSolvers/src/StokesBlockKSPInterface.c:275-448,
 *  L/Solvers/KSPSolvers/src/BSSCR/BSSCR.c:163-247,
 *  L/Solvers/KSPSolvers/src/BSSCR/auglag-driver-DGTGD.c:64-578). */
int uwg_stokes_solve(uwg_ctx* ctx, const uwg_solve_opts* opts, double* u, double* p,
                     uwg_solve_stats* stats_h);

/* Residual norms ||f - K u - G p|| and ||h - G^T u|| (free dofs), FP64.
 * Replaces Stokes_MomentumResidual / Stokes_ContinuityResidual
 * (L/StgFEM/SLE/ProvidedSystems/StokesFlow/src/Stokes_SLE.c:204-256). */
int uwg_stokes_residuals(uwg_ctx* ctx, const double* u, const double* p, double* res_h);

/* Operator applications on full node-major vectors (Dirichlet dofs masked),
 * for tests and the benchmark: y = K x (FP64 or FP32), y = G p, q = G^T u. */
int uwg_apply_K64(uwg_ctx* ctx, int level, const double* x, double* y);
int uwg_apply_K32(uwg_ctx* ctx, int level, const float* x, float* y);
int uwg_apply_G(uwg_ctx* ctx, const double* p, double* y);
int uwg_apply_Gt(uwg_ctx* ctx, const double* u, double* q);

/* Midpoint RK2 advection of every particle through the velocity field
 * vel[n_nodes][dim], with the first-order fallback when the midpoint
 * evaluation fails.  *n_fallback_h / *n_failed_h count fallbacks and
 * particles whose first evaluation failed (left untouched).
 * Replaces _TimeIntegrator_Execute -> _TimeIntegrator_ExecuteRK2 ->
 * TimeIntegrand_SecondOrder with _SwarmAdvector_TimeDeriv
 * (L/StgDomain/Utils/src/TimeIntegrator.c:292-329,
 *  L/StgDomain/Utils/src/TimeIntegrand.c:249-319,441-468,
 *  L/PICellerator/MaterialPoints/src/SwarmAdvector.c:238-312). */
int uwg_rk2_advect(uwg_ctx* ctx, int64_t np, double dt, const double* vel, double* x,
                   int64_t* n_fallback_h, int64_t* n_failed_h);

/* uwg_rk2_advect / uwg_update_owners for particle coordinates stored in FP32:
 * each stored coordinate is widened to FP64, the update is computed in FP64 as
 * above, and the new position is rounded to FP32 once when stored (the same
 * reference calls; the storage precision is this library's option for large
 * swarms). */
int uwg_rk2_advect_f32(uwg_ctx* ctx, int64_t np, double dt, const double* vel, float* x,
                       int64_t* n_fallback_h, int64_t* n_failed_h);
int uwg_update_owners_f32(uwg_ctx* ctx, int64_t np, const float* x, int32_t* owner,
                          int32_t* cell_offsets, int32_t* cell_list, int64_t* n_lost_h);

/* Velocity at arbitrary points (Mesh_SearchElements + Newton + basis);
 * points outside get NaN.  Replaces FieldVariable_InterpolateValueAt
 * (L/StgFEM/Discretisation/src/FeVariable.c:389-403). */
int uwg_interpolate(uwg_ctx* ctx, int64_t n, const double* pts, const double* vel, double* out);

/* dt = 0.5 * minimum node separation / max |v|.  Replaces SwarmAdvector_MaxDt
 * (L/PICellerator/MaterialPoints/src/SwarmAdvector.c:370-387). */
int uwg_max_dt(uwg_ctx* ctx, const double* vel, double* dt_h);
/* Values [n][ncomp] and optional global gradients [n][ncomp][dim] (grad may be NULL)
 * of a nodal field with ncomp components at points [n][dim]; NaN outside the mesh.
 * Replaces FeVariable_InterpolateValueAt / FeVariable_InterpolateDerivativesAt
 * (L/StgFEM/Discretisation/src/FeVariable.c:549-599,1007-1044) behind the function
 * graph's MeshVariable and fn_gradient inputs (P/mesh/_meshvariable.py:297-327). */
int uwg_interpolate_field(uwg_ctx* ctx, int64_t n, const double* pts, const double* field, int ncomp, double* out,
                          double* grad);

/* ---- Particle deletion and creation ----------------------------------------
 * Two-step: a plan replays the reference's sequential swarm edits on the host
 * and reports the new particle count; uwg_pop_apply then writes the new
 * particle arrays (caller-allocated for np_new particles, cell offsets for
 * n_el+1) and src_h[np_new], the old index whose swarm-variable data each new
 * particle carries.  Escaped removal replaces EscapedRoutine_RemoveFromSwarm
 * (L/PICellerator/PopulationControl/src/EscapedRoutine.c:174-284, called from
 * P/swarm/_swarm.py:644); PCDVC replaces the population control of
 * _PCDVC_Calculate2D/3D (L/PICellerator/Utils/src/PCDVC.c:313-1084, the
 * non-aggressive path) behind PopulationControl.repopulate
 * (P/swarm/_population_control.py:82-93); ip_w (and, at apply, ip_xi) are the
 * uwg_dvc_weights outputs of the current cell tables. */
int uwg_pop_plan_escaped(uwg_ctx* ctx, int64_t np, const int32_t* owner, const int32_t* cell_offsets,
                         const int32_t* cell_list, int64_t* np_new_h);
int uwg_pop_plan_pcdvc(uwg_ctx* ctx, int64_t np, const int32_t* owner, const int32_t* cell_offsets,
                       const int32_t* cell_list, const double* ip_w, double split_threshold, double delete_threshold,
                       int max_splits, int max_deletions, int64_t* np_new_h, int64_t* n_split_h, int64_t* n_deleted_h);
int uwg_pop_apply(uwg_ctx* ctx, const double* ip_xi, const double* x_old, double* x_new, int32_t* owner_new,
                  int32_t* cell_offsets_new, int32_t* cell_list_new, int64_t* src_h);

/* ---- Learned warm start: BF16 tensor-core kernels of a small CNN ------------
 * No counterpart in the reference.  Device pointers; BF16 buffers as uint16_t;
 * activations NHWC.  C[m][n] (+)= sum_k A(m,k) B(k,n) (+ bias[n]) (ReLU) with
 * A(m,k) = a_trans ? A[k*lda+m] : A[m*lda+k], B(k,n) = b_trans ? B[n*ldb+k] :
 * B[k*ldb+n], FP32 accumulation; Cf (FP32) and/or Cb (BF16) outputs.  K-major A
 * and B (a_trans 0, b_trans 1) with K, lda, ldb multiples of 8 and 16-byte aligned
 * A, B run on tcgen05.mma with the accumulator in tensor memory; the other
 * layouts on mma.sync m16n8k16. */
int uwg_cnn_gemm(uwg_ctx* ctx, int M, int N, int K, const uint16_t* A, int64_t lda, int a_trans, const uint16_t* B,
                 int64_t ldb, int b_trans, float* Cf, uint16_t* Cb, int64_t ldc, const float* bias, int relu,
                 int accumulate);
/* path 0 (default): tcgen05 where the operands allow it; 1: mma.sync always. */
int uwg_cnn_set_path(uwg_ctx* ctx, int path);
/* Synchronises the stream; UWG_ERR_CUDA if a tensor-core GEMM since the last
 * check gave up a bounded wait (its output tile is then incomplete). */
int uwg_cnn_check(uwg_ctx* ctx);
/* 3x3 im2col (BF16, zero padding) and its transpose col2im (FP32). */
int uwg_cnn_im2col(uwg_ctx* ctx, int nb, int H, int W, int C, const uint16_t* x, uint16_t* col);
int uwg_cnn_col2im(uwg_ctx* ctx, int nb, int H, int W, int C, const float* col, float* out);
/* op 0 ReLU backward, 1 2x2 average pool, 2 its transpose, 3 nearest 2x upsampling,
 * 4 its transpose, 5 BF16 add, 6 FP32 -> BF16. */
int uwg_cnn_elementwise(uwg_ctx* ctx, int op, int nb, int H, int W, int C, const uint16_t* a16, const uint16_t* b16,
                        uint16_t* c16, const float* fa, float* fb);
int uwg_cnn_bias_grad(uwg_ctx* ctx, int64_t P, int C, const float* g, float* db);
/* mean-squared error over the first nout of C channels; gradient into g, loss into *loss (device). */
int uwg_cnn_mse(uwg_ctx* ctx, int64_t P, int C, int nout, const float* y, const float* t, float* g, float* loss);
int uwg_cnn_adam(uwg_ctx* ctx, int64_t n, float* w, const float* g, float* m, float* v, uint16_t* wb, float lr,
                 float b1, float b2, float eps, int step);

/* ---- SUPG advection-diffusion of a nodal scalar (Q1 meshes) ----------------
 * One time step of the explicit predictor-multicorrector with SUPG residual and
 * lumped mass.  Replaces _AdvectionDiffusionSLE_Execute for the SUPG method
 * (P/systems/_advectiondiffusion.py:995-1007 -> L/Underworld/Utils/AdvectionDiffusion/
 * src/Multicorrector.c:166-300, Residual.cpp:213-341, LumpedMassMatrixForceTerm.c:139-172).
 *   vel       [n_nodes*dim] nodal velocity, or NULL for pure diffusion
 *   kappa_q   [n_el*3^dim] diffusivity at the 3-point Gauss points of each element
 *   source_q  same layout, or NULL
 *   bc        [n_nodes] 1 = Dirichlet node, with phi = bcval and phi-dot = bcdot (NULL: 0)
 *   phi, phidot [n_nodes] advanced in place; iterations (2) and gamma (0.5) as the reference.
 *             As in the reference, the predictor phi += dt (1-gamma) phidot, phidot = 0 is
 *             applied together with the first correction, whose residual is evaluated on
 *             phi_n and phidot_n (the reference's residual reads the nodal fields, which its
 *             predictor does not touch)
 *   flux      [n_nodes] boundary-flux vector added to every residual (the NeumannCondition
 *             surface term VectorSurfaceAssemblyTerm_NA__Fn__ni, L/Underworld/Utils/src/
 *             VectorSurfaceAssemblyTerm_NA__Fn__ni.cpp:163-236), or NULL */
int uwg_advdiff_step(uwg_ctx* ctx, double dt, const double* vel, const double* kappa_q, const double* source_q,
                     const uint8_t* bc, const double* bcval, const double* bcdot, double* phi, double* phidot,
                     int iterations, double gamma, const double* flux);
/* Time-step bound of AdvectionDiffusionSLE_CalculateDt (Timestep.c:31-117): courant *
 * min(advective, diffusive); the reference's SUPG system uses courant = 0.5. */
int uwg_advdiff_max_dt(uwg_ctx* ctx, const double* vel, const double* kappa_q, double courant, double* dt_h);

/* ---- SLCN advection-diffusion (semi-Lagrangian Crank-Nicolson, Q1 meshes) ---
 * Departure values phi*: every node traced back over dt along vel (classical RK4
 * clamped to the domain) and phi interpolated there by 4^dim Lagrange cubics on
 * the reference's static stencils.  Replaces SemiLagrangianIntegrator_SolveNew
 * (L/StgFEM/Utils/src/SemiLagrangianIntegrator.c:600-653; called from
 * P/systems/_advectiondiffusion.py:740-746).  Bit-exact.  Needs >= 4 nodes per axis. */
int uwg_slcn_phistar(uwg_ctx* ctx, double dt, const double* vel, const double* phi, double* phistar);
/* Crank-Nicolson diffusion solve (M + dt/2 D) phi = (M - dt/2 D) phi* + dt int N S with
 * Dirichlet nodes eliminated; replaces the assembly terms of
 * P/systems/_advectiondiffusion.py:211-259 and its SolveLinearSystem solve (:755).
 *   kappa_q, source_q [n_el*5^dim] at the 5-point Gauss points (source_q may be NULL)
 *   bc [n_nodes] 1 = Dirichlet node (its value is phi's current value)
 *   phi in: current field (initial guess), out: solution; CG to rtol (relative
 *   residual), its_out / res_out report the iterations and final residual.
 *   flux [n_nodes] boundary-flux vector (dt times the NeumannCondition surface term,
 *   P/systems/_advectiondiffusion.py:237-248) added to the right-hand side, or NULL. */
int uwg_slcn_solve(uwg_ctx* ctx, double dt, const double* kappa_q, const double* source_q, const uint8_t* bc,
                   const double* phistar, double* phi, double rtol, int max_its, int* its_out, double* res_out,
                   const double* flux);

#ifdef __cplusplus
}
#endif
#endif
