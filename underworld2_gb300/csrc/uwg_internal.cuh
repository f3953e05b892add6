// Internal definitions shared by the CUDA translation units of libuwg.
//
// Citations are to files of the underworld2 source tree, with
//   L/ = src/underworld/libUnderworld/
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <string>
#include <vector>

#include "../../include/uwg.h"

#define UWG_MAXLEV 16

// One multigrid level of the velocity operator.  Level 0 is the finest.
struct uwg_level {
    int order;            // velocity element order of the level (2 only on level 0 of Q2 contexts)
    int nq;               // equivalent-quadrature weights per element
    int res[3];
    int64_t n_el, n_nodes, n_dof;
    double* ax[3];        // node coordinates per axis (device)
    double* W64;          // equivalent-quadrature weights [nq][n_el] (FP64)
    float* W32;           // same in FP32
    uint8_t* bc;          // [n_nodes*dim] 1 = Dirichlet dof
    double* diag64;       // operator diagonal (BC rows = 1)
    float* diag32;
    double lmax64, lmax32; // Chebyshev upper bound for D^-1 K
    uint8_t* tile_bc;     // 3D Q1: per 8x8x4 tile, 1 when the tile holds a Dirichlet dof (tiled apply)
    float* h2inv[3];      // order-1 levels: 2 / (element size) per axis index, FP32 (tiled apply)
    float2* Wdf;          // 3D Q1 level 0: W as double-float pairs (hi, lo) for the refinement residual
    // dense coarse solve (coarsest level only)
    double* cinv64;
    float* cinv32;
};

struct uwg_ctx {
    int dim, order, porder;
    int res[3];
    double minc[3], maxc[3];
    int64_t n_el, n_nodes, n_vdof, n_pdof;
    int nen, npn, nq;      // velocity nodes / pressure nodes / equivalent points per element
    int dvc_res;
    cudaStream_t stream;
    std::string err;

    // geometry
    double* ax[3];          // finest node coordinates per axis
    double min_sep;         // Mesh_GetMinimumSeparation
    double* Gref;           // reference gradient element matrix [dim*nen][npn] (device)
    double Gref_h[81 * 4];  // host copy

    // assembled state
    int nlev;
    int pnlev;              // levels of the BFBt pressure multigrid (it stops at <= 512 cells, dense below)
    uwg_level lev[UWG_MAXLEV];
    double* f;              // velocity rhs [n_vdof] (BC lifted)
    double* h;              // pressure rhs [n_pdof]
    double* fe;             // element force [n_el][dim*nen]
    double* Shat;           // Schur preconditioner element blocks [n_el][npn*npn]
    double* Mp;             // pressure mass (compressibility) element blocks, or null
    uint8_t* bc;            // finest BC mask (alias of lev[0].bc)
    double* bcval;          // Dirichlet values [n_vdof]
    bool assembled;
    bool compressible;      // the last assembly had a pressure block C (fn_one_on_lambda)
    int64_t asm_gen;        // assemblies so far (cached operator-derived data compares against it)

    // scratch
    void* red;              // reduction scratch (double[4096])
    double* red_host;       // pinned host mirror
    std::vector<void*> ws;  // solver workspaces (freed with the context)
    double* slcn_ws;        // SLCN element matrices and CG vectors (grown on demand)
    void* pop;              // pending population plan (uwg_population.cu)
    double* q2_ke;          // 3D Q2: packed FP64 element matrices [n_el][3321] for the FP64 apply
    float2* q2_ke_df;       // the same as double-float pairs (hi, lo), for the refinement residuals
    size_t slcn_ws_bytes;
    int32_t* cnn_flag;      // CNN GEMM status word (device; set by a tensor-core GEMM whose wait gave up)
    int cnn_path;           // CNN GEMM: 0 tcgen05 where the operands allow it, 1 always mma.sync
};

// Error helpers --------------------------------------------------------------
int uwg_set_error(uwg_ctx* c, int code, const std::string& msg);
void uwg_pop_free(uwg_ctx* c);
#define UWG_CUDA(c, call)                                                                   \
    do {                                                                                     \
        cudaError_t _e = (call);                                                             \
        if (_e != cudaSuccess)                                                               \
            return uwg_set_error((c), UWG_ERR_CUDA,                                          \
                                 std::string(#call) + ": " + cudaGetErrorString(_e));        \
    } while (0)

// Device helpers ---------------------------------------------------------------
// Num_Approx (L/StGermain/Base/Foundation/src/Numerics.c:17-22)
__device__ __forceinline__ bool uwg_num_approx(double var, double val) {
    return var >= val - 1e-12 && var <= val + 1e-12;
}

// Host-side launch helpers implemented in the .cu files -------------------------
int uwg_particles_init(uwg_ctx* c);
int uwg_ops_init(uwg_ctx* c);

// Vector kernels (uwg_ops.cu)
template <typename T> void uwg_axpy(cudaStream_t s, int64_t n, T a, const T* x, T* y);
template <typename T> void uwg_fill(cudaStream_t s, int64_t n, T v, T* y);
