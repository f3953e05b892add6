// Crank-Nicolson diffusion step of SLCN advection-diffusion on a Q1 mesh: the
// linear system the reference's _SLCN_AdvectionDiffusion assembles
// (P/systems/_advectiondiffusion.py:211-259) and hands to SolveLinearSystem,
//   (M + dt/2 D) phi = (M - dt/2 D) phi* + dt int N S,
// with M the mass matrix (MatrixAssemblyTerm_NA__NB__Fn, fn = 1), D the
// diffusion matrix (MatrixAssemblyTerm_NA_i__NB_i__Fn, fn = kappa), phi* the
// semi-Lagrangian departure values (uwg_slcn_phistar), all integrated on the
// 5-point-per-axis Gauss swarm, and Dirichlet nodes eliminated with their
// values lifted to the right-hand side.
//
// Element matrices: on an axis-aligned box d_d N_a d_d N_b = (s_a s_b / h_d^2)
// times products of 1D factors N_i N_j on the other axes, so D_e needs only the
// kappa-weighted moments of those products: 9 per direction in 3D (3 in 2D),
// sum-factorised over the Gauss points a z-plane at a time.  M_e is exact
// (products of the 1D mass matrix [2/3 1/3; 1/3 2/3] h/2).  K_e = M_e + dt/2 D_e
// is kept packed (upper triangle, structure of arrays) for the CG applies.
// The solve is Jacobi-preconditioned CG in FP64 from the current phi.
#include <algorithm>
#include <cmath>
#include <cstring>

#include "uwg_ops.cuh"

namespace {

inline unsigned nblk(int64_t n, int t = 256) { return (unsigned)((n + t - 1) / t); }

// 5-point Gauss-Legendre rule, ascending abscissae; w N_i and w N_i N_j products
__constant__ double c_w5[5];
__constant__ double c_wN[2][5];    // w_q N_i(x_q)
__constant__ double c_wP[3][5];    // w_q N0^2, w_q N0 N1, w_q N1^2

template <int DIM>
__device__ __forceinline__ void slcn_nodes(const uwg_lgeom& g, int64_t e, int64_t* nodes, double* h) {
    const int ex = (int)(e % g.res[0]), ey = (int)((e / g.res[0]) % g.res[1]);
    const int ez = DIM == 3 ? (int)(e / ((int64_t)g.res[0] * g.res[1])) : 0;
    h[0] = g.ax[0][ex + 1] - g.ax[0][ex];
    h[1] = g.ax[1][ey + 1] - g.ax[1][ey];
    h[2] = DIM == 3 ? g.ax[2][ez + 1] - g.ax[2][ez] : 1.0;
#pragma unroll
    for (int n = 0; n < (1 << DIM); n++)
        nodes[n] = (ex + (n & 1)) + (int64_t)g.nx[0] * ((ey + ((n >> 1) & 1)) + (int64_t)g.nx[1] * (ez + ((n >> 2) & 1)));
}

__device__ __forceinline__ int pidx(int a, int b, int nen) {    // packed upper triangle, a <= b
    return a * nen - a * (a - 1) / 2 + (b - a);
}

template <int DIM>
__global__ void __launch_bounds__(128) k_slcn_element(uwg_lgeom g, double half_dt, double dt,
                                                      const double* __restrict__ kappa_q,
                                                      const double* __restrict__ source_q,
                                                      const double* __restrict__ phistar,
                                                      const double* __restrict__ phi,
                                                      const uint8_t* __restrict__ bc, double* __restrict__ Kp,
                                                      double* f, double* diag) {
    constexpr int NEN = 1 << DIM, NQ = DIM == 3 ? 125 : 25, NZ = DIM == 3 ? 5 : 1;
    const int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (e >= g.n_el) return;
    int64_t nodes[NEN];
    double h[3];
    slcn_nodes<DIM>(g, e, nodes, h);
    const double detJ = DIM == 3 ? (0.5 * h[0]) * (0.5 * h[1]) * (0.5 * h[2]) : (0.5 * h[0]) * (0.5 * h[1]);
    const double* kq = kappa_q + e * NQ;
    // kappa moments: Qx[ty][tz], Qy[tx][tz], Qz[tx][ty] (2D: Qx[ty], Qy[tx])
    double Qx[3][3], Qy[3][3], Qz[3][3];
#pragma unroll
    for (int a = 0; a < 3; a++)
#pragma unroll
        for (int b = 0; b < 3; b++) Qx[a][b] = Qy[a][b] = Qz[a][b] = 0.0;
    const double* sq = source_q ? source_q + e * NQ : nullptr;
    double Se[NEN];
#pragma unroll
    for (int n = 0; n < NEN; n++) Se[n] = 0.0;
#pragma unroll 1
    for (int qz = 0; qz < NZ; qz++) {
        double kp[5][5];
#pragma unroll
        for (int qy = 0; qy < 5; qy++)
#pragma unroll
            for (int qx = 0; qx < 5; qx++) kp[qx][qy] = kq[qx + 5 * qy + 25 * qz];
        double Ry[5], Rx[5];
#pragma unroll
        for (int a = 0; a < 5; a++) {
            double sy = 0.0, sx = 0.0;
#pragma unroll
            for (int b = 0; b < 5; b++) {
                sy += c_w5[b] * kp[b][a];
                sx += c_w5[b] * kp[a][b];
            }
            Ry[a] = sy;
            Rx[a] = sx;
        }
        double Tx[3], Ty[3];
#pragma unroll
        for (int t = 0; t < 3; t++) {
            double sx = 0.0, sy = 0.0;
#pragma unroll
            for (int q = 0; q < 5; q++) {
                sx += c_wP[t][q] * Ry[q];
                sy += c_wP[t][q] * Rx[q];
            }
            Tx[t] = sx;
            Ty[t] = sy;
        }
        if (DIM == 3) {
#pragma unroll
            for (int t = 0; t < 3; t++)
#pragma unroll
                for (int u = 0; u < 3; u++) {
                    Qx[t][u] += c_wP[u][qz] * Tx[t];
                    Qy[t][u] += c_wP[u][qz] * Ty[t];
                }
            double U[3][5];
#pragma unroll
            for (int t = 0; t < 3; t++)
#pragma unroll
                for (int qy = 0; qy < 5; qy++) {
                    double s = 0.0;
#pragma unroll
                    for (int qx = 0; qx < 5; qx++) s += c_wP[t][qx] * kp[qx][qy];
                    U[t][qy] = s;
                }
#pragma unroll
            for (int t = 0; t < 3; t++)
#pragma unroll
                for (int u = 0; u < 3; u++) {
                    double s = 0.0;
#pragma unroll
                    for (int qy = 0; qy < 5; qy++) s += c_wP[u][qy] * U[t][qy];
                    Qz[t][u] += c_w5[qz] * s;
                }
        } else {
#pragma unroll
            for (int t = 0; t < 3; t++) {
                Qx[t][0] = Tx[t];
                Qy[t][0] = Ty[t];
            }
        }
        if (sq) {
            double sp[5][5];
#pragma unroll
            for (int qy = 0; qy < 5; qy++)
#pragma unroll
                for (int qx = 0; qx < 5; qx++) sp[qx][qy] = sq[qx + 5 * qy + 25 * qz];
            double sx[2][5];
#pragma unroll
            for (int i = 0; i < 2; i++)
#pragma unroll
                for (int qy = 0; qy < 5; qy++) {
                    double s = 0.0;
#pragma unroll
                    for (int qx = 0; qx < 5; qx++) s += c_wN[i][qx] * sp[qx][qy];
                    sx[i][qy] = s;
                }
#pragma unroll
            for (int i = 0; i < 2; i++)
#pragma unroll
                for (int j = 0; j < 2; j++) {
                    double s = 0.0;
#pragma unroll
                    for (int qy = 0; qy < 5; qy++) s += c_wN[j][qy] * sx[i][qy];
                    if (DIM == 3) {
                        Se[i + 2 * j] += c_wN[0][qz] * s;
                        Se[i + 2 * j + 4] += c_wN[1][qz] * s;
                    } else {
                        Se[i + 2 * j] += s;
                    }
                }
        }
    }
    const double ih2[3] = {1.0 / (h[0] * h[0]), 1.0 / (h[1] * h[1]), DIM == 3 ? 1.0 / (h[2] * h[2]) : 0.0};
    double ps[NEN], pv[NEN];
    bool isbc[NEN];
#pragma unroll
    for (int n = 0; n < NEN; n++) {
        ps[n] = phistar[nodes[n]];
        isbc[n] = bc[nodes[n]] != 0;
        pv[n] = isbc[n] ? phi[nodes[n]] : 0.0;
    }
    double fe[NEN];
#pragma unroll
    for (int n = 0; n < NEN; n++) fe[n] = dt * (Se[n] * detJ);
#pragma unroll
    for (int a = 0; a < NEN; a++) {
#pragma unroll
        for (int b = a; b < NEN; b++) {
            const int ax_ = a & 1, ay = (a >> 1) & 1, az = (a >> 2) & 1;
            const int bx = b & 1, by = (b >> 1) & 1, bz = (b >> 2) & 1;
            const double sx = ax_ == bx ? 1.0 : -1.0, sy = ay == by ? 1.0 : -1.0, sz = az == bz ? 1.0 : -1.0;
            const double mx = ax_ == bx ? (2.0 / 3.0) : (1.0 / 3.0), my = ay == by ? (2.0 / 3.0) : (1.0 / 3.0);
            const double mz = az == bz ? (2.0 / 3.0) : (1.0 / 3.0);
            double D, M;
            if (DIM == 3) {
                D = (sx * ih2[0]) * Qx[ay + by][az + bz] + (sy * ih2[1]) * Qy[ax_ + bx][az + bz] +
                    (sz * ih2[2]) * Qz[ax_ + bx][ay + by];
                M = mx * my * mz;
            } else {
                D = (sx * ih2[0]) * Qx[ay + by][0] + (sy * ih2[1]) * Qy[ax_ + bx][0];
                M = mx * my;
            }
            D *= detJ;
            M *= detJ;
            const double K = M + half_dt * D, A = M - half_dt * D;
            Kp[(int64_t)pidx(a, b, NEN) * g.n_el + e] = K;
            fe[a] += A * ps[b] - K * pv[b];
            if (b != a) fe[b] += A * ps[a] - K * pv[a];
            if (a == b && !isbc[a]) atomicAdd(&diag[nodes[a]], K);
        }
    }
#pragma unroll
    for (int n = 0; n < NEN; n++)
        if (!isbc[n]) atomicAdd(&f[nodes[n]], fe[n]);
}

// y += K_ff x over the free nodes (Dirichlet entries of x read as zero)
template <int DIM>
__global__ void __launch_bounds__(256) k_slcn_apply(uwg_lgeom g, const double* __restrict__ Kp,
                                                    const uint8_t* __restrict__ bc, const double* __restrict__ x,
                                                    double* y) {
    constexpr int NEN = 1 << DIM;
    const int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (e >= g.n_el) return;
    int64_t nodes[NEN];
    double h[3];
    slcn_nodes<DIM>(g, e, nodes, h);
    double xv[NEN], yv[NEN];
    bool isbc[NEN];
#pragma unroll
    for (int n = 0; n < NEN; n++) {
        isbc[n] = bc[nodes[n]] != 0;
        xv[n] = isbc[n] ? 0.0 : x[nodes[n]];
        yv[n] = 0.0;
    }
#pragma unroll
    for (int a = 0; a < NEN; a++)
#pragma unroll
        for (int b = a; b < NEN; b++) {
            const double K = Kp[(int64_t)pidx(a, b, NEN) * g.n_el + e];
            yv[a] += K * xv[b];
            if (b != a) yv[b] += K * xv[a];
        }
#pragma unroll
    for (int n = 0; n < NEN; n++)
        if (!isbc[n]) atomicAdd(&y[nodes[n]], yv[n]);
}

__global__ void k_slcn_jacobi(int64_t n, const uint8_t* bc, const double* r, const double* diag, double* z) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i < n) z[i] = bc[i] ? 0.0 : r[i] / diag[i];
}

bool g_init = false;

int slcn_init(uwg_ctx* c) {
    if (g_init) return UWG_OK;
    // Gauss-Legendre 5: 0, +-sqrt(5 -+ 2 sqrt(10/7)) / 3; weights 128/225, (322 +- 13 sqrt 70) / 900
    const double a = std::sqrt(5.0 - 2.0 * std::sqrt(10.0 / 7.0)) / 3.0, b = std::sqrt(5.0 + 2.0 * std::sqrt(10.0 / 7.0)) / 3.0;
    const double wa = (322.0 + 13.0 * std::sqrt(70.0)) / 900.0, wb = (322.0 - 13.0 * std::sqrt(70.0)) / 900.0;
    const double x[5] = {-b, -a, 0.0, a, b}, w[5] = {wb, wa, 128.0 / 225.0, wa, wb};
    double wN[2][5], wP[3][5];
    for (int q = 0; q < 5; q++) {
        const double n0 = 0.5 * (1.0 - x[q]), n1 = 0.5 * (1.0 + x[q]);
        wN[0][q] = w[q] * n0;
        wN[1][q] = w[q] * n1;
        wP[0][q] = w[q] * n0 * n0;
        wP[1][q] = w[q] * n0 * n1;
        wP[2][q] = w[q] * n1 * n1;
    }
    UWG_CUDA(c, cudaMemcpyToSymbol(c_w5, w, sizeof(w)));
    UWG_CUDA(c, cudaMemcpyToSymbol(c_wN, wN, sizeof(wN)));
    UWG_CUDA(c, cudaMemcpyToSymbol(c_wP, wP, sizeof(wP)));
    g_init = true;
    return UWG_OK;
}

int slcn_apply(uwg_ctx* c, const uwg_lgeom& g, const double* Kp, const uint8_t* bc, const double* x, double* y) {
    cudaMemsetAsync(y, 0, sizeof(double) * c->n_nodes, c->stream);
    if (c->dim == 3) k_slcn_apply<3><<<nblk(c->n_el), 256, 0, c->stream>>>(g, Kp, bc, x, y);
    else k_slcn_apply<2><<<nblk(c->n_el), 256, 0, c->stream>>>(g, Kp, bc, x, y);
    UWG_CUDA(c, cudaGetLastError());
    return UWG_OK;
}

int dots(uwg_ctx* c, int k, const double* const* a, const double* const* b, double* out) {
    double* dst = (double*)c->red;
    vk_dots<double>(c->stream, c->n_nodes, k, a, b, dst);
    UWG_CUDA(c, cudaMemcpyAsync(out, dst, sizeof(double) * k, cudaMemcpyDeviceToHost, c->stream));
    UWG_CUDA(c, cudaStreamSynchronize(c->stream));
    return UWG_OK;
}

}  // namespace

// One Crank-Nicolson diffusion solve of SLCN (see the file header).
//   kappa_q, source_q  [n_el * 5^dim] at the Gauss points (x fastest, ascending
//                      abscissae), source_q may be NULL
//   bc                 [n_nodes] 1 = Dirichlet node; its value is phi's current value
//   phistar            [n_nodes] departure values
//   phi                [n_nodes] in: current field (initial guess), out: solution
__global__ void k_slcn_add_flux(int64_t n, const uint8_t* bc, const double* flux, double* f) {
    int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i < n && !bc[i]) f[i] += flux[i];
}

extern "C" int uwg_slcn_solve(uwg_ctx* c, double dt, const double* kappa_q, const double* source_q,
                              const uint8_t* bc, const double* phistar, double* phi, double rtol, int max_its,
                              int* its_out, double* res_out, const double* flux) {
    if (!c || !kappa_q || !bc || !phistar || !phi || !(dt >= 0.0) || !(rtol > 0.0) || max_its < 0)
        return uwg_set_error(c, UWG_ERR_ARG, "uwg_slcn_solve: bad argument");
    if (c->order != 1) return uwg_set_error(c, UWG_ERR_ARG, "SLCN diffusion is provided on Q1 meshes");
    int rc = slcn_init(c);
    if (rc) return rc;
    const int nen = 1 << c->dim, np = nen * (nen + 1) / 2;
    const int64_t n = c->n_nodes;
    const size_t need = sizeof(double) * ((size_t)np * c->n_el + 6 * (size_t)n);
    if (c->slcn_ws_bytes < need) {
        if (c->slcn_ws) cudaFree(c->slcn_ws);
        c->slcn_ws = nullptr;
        c->slcn_ws_bytes = 0;
        UWG_CUDA(c, cudaMalloc((void**)&c->slcn_ws, need));
        c->slcn_ws_bytes = need;
    }
    double* Kp = c->slcn_ws;
    double* f = Kp + (size_t)np * c->n_el;
    double *diag = f + n, *r = diag + n, *z = r + n, *p = z + n, *q = p + n;
    uwg_lgeom g = uwg_level_geom(c, 0);
    UWG_CUDA(c, cudaMemsetAsync(f, 0, sizeof(double) * 2 * n, c->stream));   // f, diag
    if (c->dim == 3)
        k_slcn_element<3><<<nblk(c->n_el, 128), 128, 0, c->stream>>>(g, 0.5 * dt, dt, kappa_q, source_q, phistar, phi,
                                                                      bc, Kp, f, diag);
    else
        k_slcn_element<2><<<nblk(c->n_el, 128), 128, 0, c->stream>>>(g, 0.5 * dt, dt, kappa_q, source_q, phistar, phi,
                                                                      bc, Kp, f, diag);
    UWG_CUDA(c, cudaGetLastError());
    if (flux) {
        k_slcn_add_flux<<<nblk(n), 256, 0, c->stream>>>(n, bc, flux, f);
        UWG_CUDA(c, cudaGetLastError());
    }
    // r = f - K x0, z = D^-1 r, p = z
    if ((rc = slcn_apply(c, g, Kp, bc, phi, q))) return rc;
    vk_copy<double>(c->stream, n, f, r);
    vk_axpy<double>(c->stream, n, -1.0, q, r);
    k_slcn_jacobi<<<nblk(n), 256, 0, c->stream>>>(n, bc, r, diag, z);
    vk_copy<double>(c->stream, n, z, p);
    double h2[2];
    {
        const double* a[2] = {r, r};
        const double* b[2] = {z, r};
        if ((rc = dots(c, 2, a, b, h2))) return rc;
    }
    double bn2;
    {
        const double* a[1] = {f};
        if ((rc = dots(c, 1, a, a, &bn2))) return rc;
    }
    double bn = std::sqrt(bn2);
    if (bn == 0.0) bn = std::sqrt(h2[1]);
    double rz = h2[0], rn = std::sqrt(h2[1]);
    int it = 0;
    while (it < max_its && rn > rtol * bn) {
        if ((rc = slcn_apply(c, g, Kp, bc, p, q))) return rc;
        double pq;
        {
            const double* a[1] = {p};
            const double* b[1] = {q};
            if ((rc = dots(c, 1, a, b, &pq))) return rc;
        }
        if (!(pq > 0.0)) return uwg_set_error(c, UWG_ERR_NAN, "uwg_slcn_solve: CG breakdown (p.Kp <= 0)");
        const double alpha = rz / pq;
        vk_axpy<double>(c->stream, n, alpha, p, phi);
        vk_axpy<double>(c->stream, n, -alpha, q, r);
        k_slcn_jacobi<<<nblk(n), 256, 0, c->stream>>>(n, bc, r, diag, z);
        {
            const double* a[2] = {r, r};
            const double* b[2] = {z, r};
            if ((rc = dots(c, 2, a, b, h2))) return rc;
        }
        const double beta = h2[0] / rz;
        rz = h2[0];
        rn = std::sqrt(h2[1]);
        vk_axpby<double>(c->stream, n, 1.0, z, beta, p);
        it++;
        if (!std::isfinite(rn)) return uwg_set_error(c, UWG_ERR_NAN, "uwg_slcn_solve: non-finite residual");
    }
    UWG_CUDA(c, cudaGetLastError());
    if (its_out) *its_out = it;
    if (res_out) *res_out = bn > 0.0 ? rn / bn : rn;
    if (rn > rtol * bn) return uwg_set_error(c, UWG_ERR_NOT_CONVERGED, "uwg_slcn_solve: CG hit its iteration cap");
    return UWG_OK;
}
