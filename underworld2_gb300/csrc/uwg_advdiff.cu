// SUPG advection-diffusion of a nodal scalar on the Q1 velocity mesh: the
// explicit predictor-multicorrector of the reference's AdvDiffMulticorrector
// (L/Underworld/Utils/AdvectionDiffusion/src/Multicorrector.c:166-300) with the
// residual of AdvDiffResidualForceTerm (Residual.cpp:213-341), the upwind
// diffusivity of Brooks & Hughes 1982 (Residual.cpp:416-506, the doubly
// asymptotic xi of :580-587 that the Python interface selects), the lumped mass of LumpedMassMatrixForceTerm.c:139-172 and the
// time-step bound of Timestep.c:31-117.  Integration is the default Gauss
// swarm: 3 points per axis.
//
// One thread per element assembles its residual (sum-factorised over the
// tensor Gauss points) and scatters it with FP64 atomics; the vector updates
// are element-free.  Dirichlet nodes are left out
// of every update (the reference removes them from its equation numbering).
//
// Order of a step, as the reference's _AdvDiffMulticorrector_Solve runs it:
// Dirichlet values go onto phi and phi-dot; the predictor acts on the
// reference's solution vectors only while its residual reads the nodal fields,
// so the first residual sees phi_n and phidot_n from before the predictor.  The
// first correction therefore applies predictor and corrector together
// (k_supg_predict_correct); later ones are plain correctors.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "uwg_geom.cuh"
#include "uwg_ops.cuh"

namespace {

inline unsigned nblk(int64_t n, int t = 256) { return (unsigned)((n + t - 1) / t); }

#define SUPG_MIN_DIFFUSIVITY 1.0e-20
#define SUPG_ISQRT15 0.25819888974716112567

// Gauss-Legendre 3-point rule on [-1, 1]
__constant__ double c_gx[3] = {-0.7745966692414834, 0.0, 0.7745966692414834};
__constant__ double c_gw[3] = {0.5555555555555556, 0.8888888888888888, 0.5555555555555556};

// Upwind parameter xi(alpha): the doubly asymptotic approximation of
// coth(alpha) - 1/alpha (Brooks & Hughes 1982, eq. 3.3.1), the one the reference's
// Python interface selects for its SUPG term ("UpwindXiFunction" =
// "DoublyAsymptoticAssumption", P/systems/sle/_assemblyterm.py:388;
// Residual.cpp:580-587)
__device__ __forceinline__ double upwind_xi(double pe) {
    if (pe <= -3.0) return -1.0;
    if (pe <= 3.0) return 0.33333333333333 * pe;
    return 1.0;
}

template <int DIM>
__device__ __forceinline__ void elem_nodes(const uwg_lgeom& g, int64_t e, int* ex, int64_t* nodes, double* h) {
    ex[0] = (int)(e % g.res[0]);
    ex[1] = (int)((e / g.res[0]) % g.res[1]);
    ex[2] = DIM == 3 ? (int)(e / ((int64_t)g.res[0] * g.res[1])) : 0;
    for (int d = 0; d < DIM; d++) h[d] = g.ax[d][ex[d] + 1] - g.ax[d][ex[d]];
    for (int n = 0; n < (1 << DIM); n++) {
        const int i = n & 1, j = (n >> 1) & 1, k = (n >> 2) & 1;
        nodes[n] = (ex[0] + i) + (int64_t)g.nx[0] * ((ex[1] + j) + (int64_t)g.nx[1] * (DIM == 3 ? ex[2] + k : 0));
    }
}

// Residual of one element, sum-factorised over the 3^DIM tensor Gauss points.
// On an axis-aligned box the Q1 shape functions are products of the 1D
// N0 = (1 - g)/2, N1 = (1 + g)/2, and their global derivatives are
// +-1/h_d times the other axes' 1D factors.  So the nodal fields are
// interpolated to the points axis by axis (z plane, y line, x point), and the
// per-point terms
//   s_q = -w_q detJ total_q,
//   w_q = -w_q detJ ((upwind total_q / |v_q|^2) v_q + kappa_q grad phi_q)
// are projected back by the transposed contraction:
//   R_n = sum_q s_q N_n(q) + w_q . grad N_n(q)
// which is the reference's sum_q -factor (supgN_n total + kappa GNx_n . grad)
// regrouped.  The lumped mass sum_q N_n(q) sum_m N_m(q) w_q detJ equals detJ
// exactly (partition of unity; sum_g w_g N(g) = 1 on each axis).  The FP64
// pipe bounds this kernel, so the regrouping is what sets its speed.
template <int DIM>
__global__ void __launch_bounds__(128) k_supg_residual(uwg_lgeom g, const double* __restrict__ vel,
                                                       const double* __restrict__ phi,
                                                       const double* __restrict__ phidot,
                                                       const double* __restrict__ kappa_q,
                                                       const double* __restrict__ source_q,
                                                       const uint8_t* __restrict__ bc, int pure_diffusion, double* R,
                                                       double* Mlump) {
    constexpr int NEN = 1 << DIM, NQ = DIM == 3 ? 27 : 9, NZ = DIM == 3 ? 3 : 1;
    int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (e >= g.n_el) return;
    int ex[3];
    int64_t nodes[NEN];
    double h[3] = {1.0, 1.0, 1.0};
    elem_nodes<DIM>(g, e, ex, nodes, h);
    double v[NEN][DIM], ph[NEN], pd[NEN];
#pragma unroll
    for (int n = 0; n < NEN; n++) {
#pragma unroll
        for (int d = 0; d < DIM; d++) v[n][d] = vel ? vel[nodes[n] * DIM + d] : 0.0;
        ph[n] = phi[nodes[n]];
        pd[n] = phidot[nodes[n]];
    }
    const double* kq = kappa_q + e * NQ;
    const double* sq = source_q ? source_q + e * NQ : nullptr;
    // upwind diffusivity from the element-average diffusivity and the centre velocity
    double kavg = 0.0;
#pragma unroll
    for (int q = 0; q < NQ; q++) kavg += kq[q];
    kavg /= (double)NQ;
    if (kavg < SUPG_MIN_DIFFUSIVITY) kavg = SUPG_MIN_DIFFUSIVITY;
    double upwind = 0.0;
#pragma unroll
    for (int d = 0; d < DIM; d++) {
        double vc = 0.0;
#pragma unroll
        for (int n = 0; n < NEN; n++) vc += v[n][d];
        vc *= 1.0 / NEN;
        const double L = fabs(h[d]);
        upwind += upwind_xi(vc * L / (2.0 * kavg)) * vc * L;
    }
    upwind *= SUPG_ISQRT15;
    const bool perturb = !pure_diffusion && !(fabs(upwind) < SUPG_MIN_DIFFUSIVITY);
    const double detJ = DIM == 3 ? (0.5 * h[0]) * (0.5 * h[1]) * (0.5 * h[2]) : (0.5 * h[0]) * (0.5 * h[1]);
    double ih[3];
#pragma unroll
    for (int d = 0; d < DIM; d++) ih[d] = 0.5 * (2.0 / h[d]);
    double t1[3], w1[3];
#pragma unroll
    for (int a = 0; a < 3; a++) {
        t1[a] = 0.5 * (1.0 + c_gx[a]);
        w1[a] = c_gw[a];
    }
    // projected residual per node: D (from s and w_x, w_y), E (from w_z) per (i, j) in the plane
    double Re[NEN];
#pragma unroll
    for (int n = 0; n < NEN; n++) Re[n] = 0.0;
#pragma unroll
    for (int qk = 0; qk < NZ; qk++) {
        // plane values at (i, j): nodal fields interpolated in z, and d/dz phi
        double pv[4][DIM], pph[4], ppd[4], pdz[4];
        const double tz = t1[qk];
#pragma unroll
        for (int p = 0; p < 4; p++) {
            if (DIM == 3) {
#pragma unroll
                for (int d = 0; d < DIM; d++) pv[p][d] = v[p][d] + (v[p + 4][d] - v[p][d]) * tz;
                pph[p] = ph[p] + (ph[p + 4] - ph[p]) * tz;
                ppd[p] = pd[p] + (pd[p + 4] - pd[p]) * tz;
                pdz[p] = (ph[p + 4] - ph[p]) * ih[DIM - 1];
            } else {
#pragma unroll
                for (int d = 0; d < DIM; d++) pv[p][d] = v[p][d];
                pph[p] = ph[p];
                ppd[p] = pd[p];
                pdz[p] = 0.0;
            }
        }
        double D[4] = {0.0, 0.0, 0.0, 0.0}, E[4] = {0.0, 0.0, 0.0, 0.0};
        const double wk = (DIM == 3 ? w1[qk] : 1.0) * detJ;
#pragma unroll
        for (int qj = 0; qj < 3; qj++) {
            const double ty = t1[qj];
            // line values at i = 0, 1
            double lv[2][DIM], lpd[2], ldz[2], ldy[2], lph[2];
#pragma unroll
            for (int i = 0; i < 2; i++) {
#pragma unroll
                for (int d = 0; d < DIM; d++) lv[i][d] = pv[i][d] + (pv[i + 2][d] - pv[i][d]) * ty;
                lph[i] = pph[i] + (pph[i + 2] - pph[i]) * ty;
                lpd[i] = ppd[i] + (ppd[i + 2] - ppd[i]) * ty;
                ldz[i] = pdz[i] + (pdz[i + 2] - pdz[i]) * ty;
                ldy[i] = (pph[i + 2] - pph[i]) * ih[1];
            }
            const double dx = (lph[1] - lph[0]) * ih[0];
            double dv[DIM];
#pragma unroll
            for (int d = 0; d < DIM; d++) dv[d] = lv[1][d] - lv[0][d];
            const double dpd = lpd[1] - lpd[0], ddz = ldz[1] - ldz[0], ddy = ldy[1] - ldy[0];
            const double wjk = w1[qj] * wk;
            double s0 = 0.0, s1 = 0.0, sx = 0.0, y0 = 0.0, y1 = 0.0, z0 = 0.0, z1 = 0.0;
#pragma unroll
            for (int qi = 0; qi < 3; qi++) {
                const double tx = t1[qi], ux = 1.0 - tx;
                const int q = qi + 3 * qj + 9 * qk;
                double vq[3] = {0.0, 0.0, 0.0};
#pragma unroll
                for (int d = 0; d < DIM; d++) vq[d] = lv[0][d] + dv[d] * tx;
                const double gy = ldy[0] + ddy * tx;
                const double gz = DIM == 3 ? ldz[0] + ddz * tx : 0.0;
                const double factor = w1[qi] * wjk;
                const double fk = factor * kq[q];
                double wx = fk * dx, wy = fk * gy, wz = fk * gz;
                double sv = 0.0;
                if (!pure_diffusion) {
                    double total = lpd[0] + dpd * tx;
                    total += vq[0] * dx + vq[1] * gy + (DIM == 3 ? vq[2] * gz : 0.0);
                    if (sq) total -= sq[q];
                    const double ftot = factor * total;
                    sv = ftot;
                    if (perturb) {
                        const double udotu = vq[0] * vq[0] + vq[1] * vq[1] + (DIM == 3 ? vq[2] * vq[2] : 0.0);
                        const double cs = ftot * (upwind / udotu);
                        wx += cs * vq[0];
                        wy += cs * vq[1];
                        if (DIM == 3) wz += cs * vq[2];
                    }
                }
                s0 += sv * ux;
                s1 += sv * tx;
                sx += wx;
                y0 += wy * ux;
                y1 += wy * tx;
                z0 += wz * ux;
                z1 += wz * tx;
            }
            // x-projected: A_i (s and w_x), B_i (w_y), C_i (w_z); then project in y
            const double A[2] = {s0 - sx * ih[0], s1 + sx * ih[0]};
            const double B[2] = {y0, y1}, C[2] = {z0, z1};
            const double uy = 1.0 - ty;
#pragma unroll
            for (int i = 0; i < 2; i++) {
                D[i] += A[i] * uy - B[i] * ih[1];
                D[i + 2] += A[i] * ty + B[i] * ih[1];
                E[i] += C[i] * uy;
                E[i + 2] += C[i] * ty;
            }
        }
        if (DIM == 3) {
            const double uz = 1.0 - tz;
#pragma unroll
            for (int p = 0; p < 4; p++) {
                Re[p] += D[p] * uz - E[p] * ih[2];
                Re[p + 4] += D[p] * tz + E[p] * ih[2];
            }
        } else {
#pragma unroll
            for (int p = 0; p < 4; p++) Re[p] += D[p];
        }
    }
#pragma unroll
    for (int n = 0; n < NEN; n++) {
        if (bc[nodes[n]]) continue;
        atomicAdd(&R[nodes[n]], -Re[n]);
        if (Mlump) atomicAdd(&Mlump[nodes[n]], detJ);
    }
}

__global__ void k_supg_predict(int64_t n, const uint8_t* bc, const double* bcval, const double* bcdot, double f,
                               double* phi, double* phidot) {
    int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    if (bc[i]) {
        phi[i] = bcval[i];
        phidot[i] = bcdot ? bcdot[i] : 0.0;
        return;
    }
    phi[i] += f * phidot[i];
    phidot[i] = 0.0;
}

// Dirichlet values onto both fields (FeVariable_ApplyBCs on phi and phi-dot)
__global__ void k_supg_bc(int64_t n, const uint8_t* bc, const double* bcval, const double* bcdot, double* phi,
                          double* phidot) {
    int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n || !bc[i]) return;
    phi[i] = bcval[i];
    phidot[i] = bcdot ? bcdot[i] : 0.0;
}

// First correction with the predictor: d = R / M,
// phi = (phi_n + fp phidot_n) + fc d, phidot = d.  flux as k_supg_correct.
__global__ void k_supg_predict_correct(int64_t n, const uint8_t* bc, const double* R, const double* flux,
                                       const double* M, double fp, double fc, double* phi, double* phidot) {
    int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n || bc[i]) return;
    const double d = (flux ? R[i] + flux[i] : R[i]) / M[i];
    const double p = phi[i] + fp * phidot[i];
    phi[i] = p + fc * d;
    phidot[i] = d;
}

// flux: the boundary-flux vector added to the residual, or NULL
__global__ void k_supg_correct(int64_t n, const uint8_t* bc, const double* R, const double* flux, const double* M,
                               double f, double* phi, double* phidot) {
    int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n || bc[i]) return;
    const double d = (flux ? R[i] + flux[i] : R[i]) / M[i];
    phi[i] += f * d;
    phidot[i] += d;
}

// time-step bounds: per node min_d |minsep_d / v_d| (advective) and, per Gauss
// point, the diffusivity maximum; both reduced through the bit patterns of
// non-negative doubles
__global__ void k_supg_dt(int64_t n_nodes, int dim, const double* vel, double s0, double s1, double s2,
                          int64_t nk, const double* kappa_q, unsigned long long* out) {
    int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i < n_nodes && vel) {
        double t = HUGE_VAL;
        const double sep[3] = {s0, s1, s2};
        for (int d = 0; d < dim; d++) {
            const double vd = vel[i * dim + d];
            if (vd == 0.0) continue;
            t = fmin(t, fabs(sep[d] / vd));
        }
        if (t < HUGE_VAL) atomicMin(&out[0], (unsigned long long)__double_as_longlong(t));
    }
    if (i < nk) atomicMax(&out[1], (unsigned long long)__double_as_longlong(fmax(kappa_q[i], 0.0)));
}

}  // namespace

// Courant-limited time step of the reference's AdvectionDiffusionSLE_CalculateDt
// (Timestep.c:31-117): courant * min(min_nodes,d |minsep_d / v_d|, minsep^2 / max kappa).
extern "C" int uwg_advdiff_max_dt(uwg_ctx* c, const double* vel, const double* kappa_q, double courant,
                                  double* dt_out) {
    if (!c || !kappa_q || !dt_out) return uwg_set_error(c, UWG_ERR_ARG, "uwg_advdiff_max_dt: bad argument");
    double sep[3] = {HUGE_VAL, HUGE_VAL, HUGE_VAL};
    for (int d = 0; d < c->dim; d++) {
        std::vector<double> ax(c->res[d] + 1);
        UWG_CUDA(c, cudaMemcpy(ax.data(), c->ax[d], sizeof(double) * ax.size(), cudaMemcpyDeviceToHost));
        for (size_t k = 0; k + 1 < ax.size(); k++) sep[d] = std::min(sep[d], std::fabs(ax[k + 1] - ax[k]));
    }
    double minsep = std::min(sep[0], std::min(sep[1], sep[2]));
    unsigned long long* out = (unsigned long long*)c->red;
    unsigned long long init[2] = {(unsigned long long)0x7FF0000000000000ull, 0ull};   // +inf, 0
    UWG_CUDA(c, cudaMemcpyAsync(out, init, sizeof(init), cudaMemcpyHostToDevice, c->stream));
    const int64_t nk = c->n_el * (c->dim == 3 ? 27 : 9);
    const int64_t nt = std::max<int64_t>(c->n_nodes, nk);
    k_supg_dt<<<nblk(nt), 256, 0, c->stream>>>(c->n_nodes, c->dim, vel, sep[0], sep[1], sep[2], nk, kappa_q, out);
    unsigned long long h[2];
    UWG_CUDA(c, cudaGetLastError());
    UWG_CUDA(c, cudaMemcpyAsync(h, out, sizeof(h), cudaMemcpyDeviceToHost, c->stream));
    UWG_CUDA(c, cudaStreamSynchronize(c->stream));
    double adv, kmax;
    std::memcpy(&adv, &h[0], 8);
    std::memcpy(&kmax, &h[1], 8);
    const double diff = kmax > 0.0 ? minsep * minsep / kmax : HUGE_VAL;
    *dt_out = courant * std::min(vel ? adv : HUGE_VAL, diff);
    return UWG_OK;
}

// One time step of SUPG advection-diffusion (see the file header).
//   vel      [n_nodes*dim] nodal velocity (NULL: pure diffusion)
//   kappa_q  [n_el*3^dim] diffusivity at the Gauss points; source_q likewise or NULL
//   bc       [n_nodes] 1 = Dirichlet node; bcval, bcdot its phi and phi-dot values
extern "C" int uwg_advdiff_step(uwg_ctx* c, double dt, const double* vel, const double* kappa_q,
                                const double* source_q, const uint8_t* bc, const double* bcval, const double* bcdot,
                                double* phi, double* phidot, int iterations, double gamma, const double* flux) {
    if (!c || !kappa_q || !bc || !bcval || !phi || !phidot || iterations < 0 || !(dt >= 0.0))
        return uwg_set_error(c, UWG_ERR_ARG, "uwg_advdiff_step: bad argument");
    if (c->order != 1) return uwg_set_error(c, UWG_ERR_ARG, "advection-diffusion is provided on Q1 meshes");
    const int64_t n = c->n_nodes;
    uwg_lgeom g = uwg_level_geom(c, 0);
    double *R = nullptr, *M = nullptr;
    UWG_CUDA(c, cudaMallocAsync((void**)&R, sizeof(double) * n, c->stream));
    UWG_CUDA(c, cudaMallocAsync((void**)&M, sizeof(double) * n, c->stream));
    if (iterations == 0)        // predictor only
        k_supg_predict<<<nblk(n), 256, 0, c->stream>>>(n, bc, bcval, bcdot, dt * (1.0 - gamma), phi, phidot);
    else
        k_supg_bc<<<nblk(n), 256, 0, c->stream>>>(n, bc, bcval, bcdot, phi, phidot);
    cudaError_t err = cudaGetLastError();
    for (int it = 0; it < iterations && err == cudaSuccess; it++) {
        cudaMemsetAsync(R, 0, sizeof(double) * n, c->stream);
        if (it == 0) cudaMemsetAsync(M, 0, sizeof(double) * n, c->stream);
        if (c->dim == 3)
            k_supg_residual<3><<<nblk(c->n_el, 128), 128, 0, c->stream>>>(g, vel, phi, phidot, kappa_q, source_q, bc,
                                                                          vel ? 0 : 1, R, it == 0 ? M : nullptr);
        else
            k_supg_residual<2><<<nblk(c->n_el, 128), 128, 0, c->stream>>>(g, vel, phi, phidot, kappa_q, source_q, bc,
                                                                          vel ? 0 : 1, R, it == 0 ? M : nullptr);
        if (it == 0)
            k_supg_predict_correct<<<nblk(n), 256, 0, c->stream>>>(n, bc, R, flux, M, dt * (1.0 - gamma),
                                                                   dt * gamma, phi, phidot);
        else
            k_supg_correct<<<nblk(n), 256, 0, c->stream>>>(n, bc, R, flux, M, dt * gamma, phi, phidot);
        err = cudaGetLastError();
    }
    cudaFreeAsync(R, c->stream);
    cudaFreeAsync(M, c->stream);
    if (err != cudaSuccess) return uwg_set_error(c, UWG_ERR_CUDA, cudaGetErrorString(err));
    return UWG_OK;
}
