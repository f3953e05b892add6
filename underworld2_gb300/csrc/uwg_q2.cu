// 2D Q2/dPc1 operators: biquadratic velocity, linear discontinuous pressure.
//
// Level 0 of a Q2 context is the Q2 mesh; level 1 is the Q1 mesh on the same
// elements (the p-coarsening of the velocity multigrid) and the levels below
// it are the usual halved Q1 meshes.
//
// * Viscous operator.  On affine elements every entry of the PIC integrand
//   B^T D(eta) B of a Q2 element is a polynomial of degree <= 4 per axis in
//   the local coordinates, so 5-point tensor Lagrange interpolation on
//   {-1,-1/2,0,1/2,1}^2 reproduces it exactly:
//       W_j = sum_q eta_q w_q detJ L_j(xi_q),   K_e = sum_j W_j F(xi_j)
//   (25 weights per element instead of an 18x18 matrix; the same identity as
//   the 3-point weights of Q1).  K_e is applied sum-factorised on the 5x5 grid.
//   The Galerkin Q1 operator P^T K P of the same element is the Q1 PIC
//   integral, so level 1 takes the 3-point weights of the same particles.
// * Gradient.  G_e[(A,i)][k] = -int dN_A/dx_i M_k (GradientStiffnessMatrixTerm.c
//   :189-218) with the dPc1 basis M of BilinearInnerElType.c:169-179; on a
//   Cartesian element it is -(h_j/2) times a reference integral, tabulated once.
// * Schur preconditioner.  The reference's Uzawa term S^_e = G_e^T diag(K_e)^-1 G_e
//   (UzawaPreconditionerTerm.c:124-207) is a 3x3 block per element for dPc1;
//   PETSc's ILU(0) of a block-diagonal matrix is its exact inverse, which is
//   what is stored.
#include <cmath>

#include "uwg_ops.cuh"

namespace {

inline unsigned nblk(int64_t n, int t = 256) { return (unsigned)((n + t - 1) / t); }

// 1D quadratic basis on nodes {-1, 0, 1} and its derivative at the five
// points {-1, -1/2, 0, 1/2, 1}: B5[p][a] = N_a(s_p), D5[p][a] = N_a'(s_p)
__constant__ double c_B5[5][3] = {{1.0, 0.0, 0.0}, {0.375, 0.75, -0.125}, {0.0, 1.0, 0.0},
                                  {-0.125, 0.75, 0.375}, {0.0, 0.0, 1.0}};
__constant__ double c_D5[5][3] = {{-1.5, 2.0, -0.5}, {-1.0, 1.0, 0.0}, {-0.5, 0.0, 0.5},
                                  {0.0, -1.0, 1.0}, {0.5, -2.0, 1.5}};
// reference gradient integrals: c_GR[i][A][k] = int dN_A/dxi_i M_k over [-1,1]^2
__constant__ double c_GR[2][9][3];

__device__ __forceinline__ void q2_elem(const uwg_lgeom& g, int64_t e, int64_t* nodes, double& hx, double& hy) {
    int ex = (int)(e % g.res[0]), ey = (int)(e / g.res[0]);
    hx = g.ax[0][2 * ex + 2] - g.ax[0][2 * ex];
    hy = g.ax[1][2 * ey + 2] - g.ax[1][2 * ey];
    for (int b = 0; b < 3; b++)
        for (int a = 0; a < 3; a++) nodes[a + 3 * b] = (2 * ex + a) + (int64_t)g.nx[0] * (2 * ey + b);
}

// 1D Lagrange bases: 3 points {-1,0,1} and 5 points {-1,-1/2,0,1/2,1}
__device__ __forceinline__ void lag3q(double s, double* l) {
    l[0] = 0.5 * s * (s - 1.0);
    l[1] = 1.0 - s * s;
    l[2] = 0.5 * s * (s + 1.0);
}
__device__ __forceinline__ void lag5(double s, double* l) {
    const double n[5] = {-1.0, -0.5, 0.0, 0.5, 1.0};
#pragma unroll
    for (int j = 0; j < 5; j++) {
        double v = 1.0;
#pragma unroll
        for (int k = 0; k < 5; k++)
            if (k != j) v *= (s - n[k]) / (n[j] - n[k]);
        l[j] = v;
    }
}

// PIC assembly, one thread per element: 25 Q2 weights, 9 Q1 weights (level 1)
// and the body force on the Q2 nodes.
__global__ void k_assemble_q2(uwg_lgeom g, const int32_t* off, const int32_t* list, const double* ip_xi,
                              const double* ip_w, const double* eta_p, const double* body_p, double* W25,
                              double* W9, double* f) {
    int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (e >= g.n_el) return;
    int64_t nodes[9];
    double hx, hy;
    q2_elem(g, e, nodes, hx, hy);
    const double detJ = (hx * 0.5) * (hy * 0.5);
    double w25[25], w9[9], fe[18];
    for (int j = 0; j < 25; j++) w25[j] = 0.0;
    for (int j = 0; j < 9; j++) w9[j] = 0.0;
    for (int j = 0; j < 18; j++) fe[j] = 0.0;
    for (int32_t s = off[e]; s < off[e + 1]; s++) {
        int32_t p = list[s];
        const double xi = ip_xi[(int64_t)s * 2], et = ip_xi[(int64_t)s * 2 + 1];
        const double wd = ip_w[s] * detJ, c = eta_p[p] * wd;
        double l5x[5], l5y[5], l3x[3], l3y[3];
        lag5(xi, l5x);
        lag5(et, l5y);
        lag3q(xi, l3x);
        lag3q(et, l3y);
        for (int q = 0; q < 5; q++)
            for (int pp = 0; pp < 5; pp++) w25[pp + 5 * q] += c * l5x[pp] * l5y[q];
        for (int q = 0; q < 3; q++)
            for (int pp = 0; pp < 3; pp++) w9[pp + 3 * q] += c * l3x[pp] * l3y[q];
        if (body_p) {
            // Q2 basis N_A = N_a(xi) N_b(eta) (the 3-point Lagrange basis)
            for (int b = 0; b < 3; b++)
                for (int a = 0; a < 3; a++)
                    for (int i = 0; i < 2; i++) fe[(a + 3 * b) * 2 + i] += wd * body_p[(int64_t)p * 2 + i] * (l3x[a] * l3y[b]);
        }
    }
    for (int j = 0; j < 25; j++) W25[(int64_t)j * g.n_el + e] = w25[j];
    for (int j = 0; j < 9; j++) W9[(int64_t)j * g.n_el + e] = w9[j];
    if (body_p)
        for (int A = 0; A < 9; A++)
            for (int i = 0; i < 2; i++) atomicAdd(&f[nodes[A] * 2 + i], fe[A * 2 + i]);
}

// y_e = K_e u_e for one Q2 element from its 25 weights (sum-factorised).
template <typename T>
__device__ __forceinline__ void q2_element(const T* __restrict__ Wp, int64_t stride, T sx, T sy, const T (&u)[9][2],
                                           T (&out)[9][2]) {
    T gx[2][5][5], gy[2][5][5];   // [c][p][q]: d u_c / dx, d u_c / dy at point (p, q)
#pragma unroll
    for (int c = 0; c < 2; c++) {
        T t[3][5], s[3][5];
#pragma unroll
        for (int a = 0; a < 3; a++)
#pragma unroll
            for (int q = 0; q < 5; q++) {
                T tv = 0, sv = 0;
#pragma unroll
                for (int b = 0; b < 3; b++) {
                    tv += (T)c_B5[q][b] * u[a + 3 * b][c];
                    sv += (T)c_D5[q][b] * u[a + 3 * b][c];
                }
                t[a][q] = tv;
                s[a][q] = sv;
            }
#pragma unroll
        for (int p = 0; p < 5; p++)
#pragma unroll
            for (int q = 0; q < 5; q++) {
                T vx = 0, vy = 0;
#pragma unroll
                for (int a = 0; a < 3; a++) {
                    vx += (T)c_D5[p][a] * t[a][q];
                    vy += (T)c_B5[p][a] * s[a][q];
                }
                gx[c][p][q] = sx * vx;
                gy[c][p][q] = sy * vy;
            }
    }
    // stresses in place: gx <- R_x, gy <- R_y
#pragma unroll
    for (int q = 0; q < 5; q++)
#pragma unroll
        for (int p = 0; p < 5; p++) {
            const T w = Wp[(int64_t)(p + 5 * q) * stride];
            const T uxx = gx[0][p][q], uxy = gy[0][p][q], uyx = gx[1][p][q], uyy = gy[1][p][q];
            const T sxx = w * (uxx + uxx), syy = w * (uyy + uyy), sxy = w * (uxy + uyx);
            gx[0][p][q] = sxx;
            gy[0][p][q] = sxy;
            gx[1][p][q] = sxy;
            gy[1][p][q] = syy;
        }
#pragma unroll
    for (int c = 0; c < 2; c++) {
        T tx[5][3], ty[5][3];
#pragma unroll
        for (int p = 0; p < 5; p++)
#pragma unroll
            for (int b = 0; b < 3; b++) {
                T a1 = 0, a2 = 0;
#pragma unroll
                for (int q = 0; q < 5; q++) {
                    a1 += (T)c_B5[q][b] * gx[c][p][q];
                    a2 += (T)c_D5[q][b] * gy[c][p][q];
                }
                tx[p][b] = a1;
                ty[p][b] = a2;
            }
#pragma unroll
        for (int b = 0; b < 3; b++)
#pragma unroll
            for (int a = 0; a < 3; a++) {
                T v1 = 0, v2 = 0;
#pragma unroll
                for (int p = 0; p < 5; p++) {
                    v1 += (T)c_D5[p][a] * tx[p][b];
                    v2 += (T)c_B5[p][a] * ty[p][b];
                }
                out[a + 3 * b][c] = sx * v1 + sy * v2;
            }
    }
}

template <typename T>
__global__ void k_applyK_q2(uwg_lgeom g, const T* __restrict__ W, const uint8_t* __restrict__ bc, bool mask_in,
                            const T* __restrict__ x, T* y) {
    int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (e >= g.n_el) return;
    int64_t nodes[9];
    double hx, hy;
    q2_elem(g, e, nodes, hx, hy);
    const T sx = (T)2 / (T)hx, sy = (T)2 / (T)hy;
    T u[9][2], out[9][2];
    bool fix[9][2];
#pragma unroll
    for (int A = 0; A < 9; A++)
#pragma unroll
        for (int c = 0; c < 2; c++) {
            int64_t dof = nodes[A] * 2 + c;
            fix[A][c] = bc[dof] != 0;
            u[A][c] = (fix[A][c] && mask_in) ? (T)0 : x[dof];
        }
    q2_element<T>(W + e, g.n_el, sx, sy, u, out);
#pragma unroll
    for (int A = 0; A < 9; A++)
#pragma unroll
        for (int c = 0; c < 2; c++)
            if (!fix[A][c]) atomicAdd(&y[nodes[A] * 2 + c], out[A][c]);
}

// G_e[(A,i)][k] of element e (18 x 3)
__device__ __forceinline__ void q2_Ge(double hx, double hy, double (&Ge)[18][3]) {
    for (int A = 0; A < 9; A++)
        for (int k = 0; k < 3; k++) {
            Ge[A * 2 + 0][k] = -(hy * 0.5) * c_GR[0][A][k];
            Ge[A * 2 + 1][k] = -(hx * 0.5) * c_GR[1][A][k];
        }
}

// diagonal of K (assembled, free dofs) and, per element, the inverse of
// S^_e = G_e^T diag(K_e)^-1 G_e
__global__ void k_diag_q2(uwg_lgeom g, const double* W, const uint8_t* bc, double* diag, double* sinv) {
    int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (e >= g.n_el) return;
    int64_t nodes[9];
    double hx, hy;
    q2_elem(g, e, nodes, hx, hy);
    const double sx = 2.0 / hx, sy = 2.0 / hy;
    double kd[9][2];
    for (int A = 0; A < 9; A++) kd[A][0] = kd[A][1] = 0.0;
    for (int q = 0; q < 5; q++)
        for (int p = 0; p < 5; p++) {
            const double w = W[(int64_t)(p + 5 * q) * g.n_el + e];
            for (int b = 0; b < 3; b++)
                for (int a = 0; a < 3; a++) {
                    const double nx = sx * c_D5[p][a] * c_B5[q][b], ny = sy * c_B5[p][a] * c_D5[q][b];
                    const double s2 = nx * nx + ny * ny;
                    kd[a + 3 * b][0] += w * (s2 + nx * nx);
                    kd[a + 3 * b][1] += w * (s2 + ny * ny);
                }
        }
    for (int A = 0; A < 9; A++)
        for (int c = 0; c < 2; c++) {
            int64_t dof = nodes[A] * 2 + c;
            if (!bc[dof]) atomicAdd(&diag[dof], kd[A][c]);
        }
    if (!sinv) return;
    double Ge[18][3];
    q2_Ge(hx, hy, Ge);
    double S[3][3];
    for (int k = 0; k < 3; k++)
        for (int l = 0; l < 3; l++) {
            double s = 0.0;
            for (int r = 0; r < 18; r++) s += Ge[r][k] * (Ge[r][l] / kd[r / 2][r % 2]);
            S[k][l] = s;
        }
    // explicit inverse of the SPD 3x3 block
    const double c00 = S[1][1] * S[2][2] - S[1][2] * S[2][1], c01 = S[1][2] * S[2][0] - S[1][0] * S[2][2],
                 c02 = S[1][0] * S[2][1] - S[1][1] * S[2][0];
    const double det = S[0][0] * c00 + S[0][1] * c01 + S[0][2] * c02;
    const double id = 1.0 / det;
    double* o = sinv + e * 9;
    o[0] = c00 * id;
    o[1] = (S[0][2] * S[2][1] - S[0][1] * S[2][2]) * id;
    o[2] = (S[0][1] * S[1][2] - S[0][2] * S[1][1]) * id;
    o[3] = c01 * id;
    o[4] = (S[0][0] * S[2][2] - S[0][2] * S[2][0]) * id;
    o[5] = (S[0][2] * S[1][0] - S[0][0] * S[1][2]) * id;
    o[6] = c02 * id;
    o[7] = (S[0][1] * S[2][0] - S[0][0] * S[2][1]) * id;
    o[8] = (S[0][0] * S[1][1] - S[0][1] * S[1][0]) * id;
}

// y += G p on free dofs (y is zeroed by the caller)
__global__ void k_applyG_q2(uwg_lgeom g, const uint8_t* bc, const double* p, double* y) {
    int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (e >= g.n_el) return;
    int64_t nodes[9];
    double hx, hy;
    q2_elem(g, e, nodes, hx, hy);
    double Ge[18][3];
    q2_Ge(hx, hy, Ge);
    const double p0 = p[e * 3], p1 = p[e * 3 + 1], p2 = p[e * 3 + 2];
    for (int r = 0; r < 18; r++) {
        int64_t dof = nodes[r / 2] * 2 + (r % 2);
        if (!bc[dof]) atomicAdd(&y[dof], Ge[r][0] * p0 + Ge[r][1] * p1 + Ge[r][2] * p2);
    }
}

// q = G^T u over free dofs (only_bc = 0) or over Dirichlet dofs (only_bc = 1)
__global__ void k_applyGt_q2(uwg_lgeom g, const uint8_t* bc, int only_bc, const double* u, double* q) {
    int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (e >= g.n_el) return;
    int64_t nodes[9];
    double hx, hy;
    q2_elem(g, e, nodes, hx, hy);
    double Ge[18][3];
    q2_Ge(hx, hy, Ge);
    double s[3] = {0.0, 0.0, 0.0};
    for (int r = 0; r < 18; r++) {
        int64_t dof = nodes[r / 2] * 2 + (r % 2);
        if ((bc[dof] != 0) != (only_bc != 0)) continue;
        const double v = u[dof];
        for (int k = 0; k < 3; k++) s[k] += Ge[r][k] * v;
    }
    for (int k = 0; k < 3; k++) q[e * 3 + k] = s[k];
}

__global__ void k_schur_pc_q2(int64_t n_el, const double* sinv, const double* r, double* z) {
    int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (e >= n_el) return;
    const double* S = sinv + e * 9;
    const double r0 = r[e * 3], r1 = r[e * 3 + 1], r2 = r[e * 3 + 2];
    z[e * 3 + 0] = S[0] * r0 + S[1] * r1 + S[2] * r2;
    z[e * 3 + 1] = S[3] * r0 + S[4] * r1 + S[5] * r2;
    z[e * 3 + 2] = S[6] * r0 + S[7] * r1 + S[8] * r2;
}

// Element matrices of one element (diagnostics): K_e column by column, G_e, S^_e
__global__ void k_element_matrices_q2(uwg_lgeom g, int64_t e, const double* W, double* Ke, double* Ge_out,
                                      double* Se) {
    int64_t nodes[9];
    double hx, hy;
    q2_elem(g, e, nodes, hx, hy);
    const double sx = 2.0 / hx, sy = 2.0 / hy;
    for (int col = 0; col < 18; col++) {
        double u[9][2], out[9][2];
        for (int A = 0; A < 9; A++) u[A][0] = u[A][1] = 0.0;
        u[col / 2][col % 2] = 1.0;
        q2_element<double>(W + e, g.n_el, sx, sy, u, out);
        for (int r = 0; r < 18; r++) Ke[r * 18 + col] = out[r / 2][r % 2];
    }
    double Ge[18][3];
    q2_Ge(hx, hy, Ge);
    for (int r = 0; r < 18; r++)
        for (int k = 0; k < 3; k++) Ge_out[r * 3 + k] = Ge[r][k];
    for (int k = 0; k < 3; k++)
        for (int l = 0; l < 3; l++) {
            double s = 0.0;
            for (int r = 0; r < 18; r++) s += Ge[r][k] * (Ge[r][l] / Ke[r * 18 + r]);
            Se[k * 3 + l] = s;
        }
}

// dPc1 basis (BilinearInnerElType.c:169-179) and the 1D quadratic basis, host side
void dpc1_host(double xi, double eta, double* M) {
    M[0] = -xi - 0.5 * eta + 0.25;
    M[1] = xi - 0.5 * eta + 0.25;
    M[2] = eta + 0.5;
}
void q2_1d_host(double s, double* N, double* D) {
    N[0] = 0.5 * s * (s - 1.0); N[1] = 1.0 - s * s; N[2] = 0.5 * s * (s + 1.0);
    D[0] = s - 0.5; D[1] = -2.0 * s; D[2] = s + 0.5;
}

}  // namespace

// ---------------------------------------------------------------------------
// Host wrappers
// ---------------------------------------------------------------------------
int uwg_q2_init(uwg_ctx* c) {
    if (c->dim == 3) return uwg_q2_3d_init(c);
    // reference gradient integrals with the 3-point Gauss rule (exact: degree <= 3 per axis)
    const double gp[3] = {-std::sqrt(0.6), 0.0, std::sqrt(0.6)}, gw[3] = {5.0 / 9.0, 8.0 / 9.0, 5.0 / 9.0};
    double GR[2][9][3] = {};
    for (int j = 0; j < 3; j++)
        for (int i = 0; i < 3; i++) {
            double Nx[3], Dx[3], Ny[3], Dy[3], M[3];
            q2_1d_host(gp[i], Nx, Dx);
            q2_1d_host(gp[j], Ny, Dy);
            dpc1_host(gp[i], gp[j], M);
            for (int b = 0; b < 3; b++)
                for (int a = 0; a < 3; a++)
                    for (int k = 0; k < 3; k++) {
                        GR[0][a + 3 * b][k] += gw[i] * gw[j] * Dx[a] * Ny[b] * M[k];
                        GR[1][a + 3 * b][k] += gw[i] * gw[j] * Nx[a] * Dy[b] * M[k];
                    }
        }
    UWG_CUDA(c, cudaMemcpyToSymbol(c_GR, GR, sizeof(GR)));
    return UWG_OK;
}

int uwg_q2_assemble(uwg_ctx* c, const int32_t* off, const int32_t* list, const double* ip_xi, const double* ip_w,
                    const double* eta_p, const double* body_p) {
    if (c->dim == 3) return uwg_q2_3d_assemble(c, off, list, ip_xi, ip_w, eta_p, body_p);
    uwg_lgeom g = uwg_level_geom(c, 0);
    vk_zero<double>(c->stream, c->n_vdof, c->f);
    k_assemble_q2<<<nblk(c->n_el, 128), 128, 0, c->stream>>>(g, off, list, ip_xi, ip_w, eta_p, body_p, c->lev[0].W64,
                                                             c->lev[1].W64, c->f);
    UWG_CUDA(c, cudaGetLastError());
    return UWG_OK;
}

template <typename T>
int uwg_q2_applyK(uwg_ctx* c, const T* x, T* y, bool mask_in) {
    if (c->dim == 3) return uwg_q2_3d_applyK<T>(c, x, y, mask_in);
    const uwg_level& L = c->lev[0];
    const T* W;
    if constexpr (sizeof(T) == 8) W = (const T*)L.W64; else W = (const T*)L.W32;
    k_applyK_q2<T><<<nblk(L.n_el, 128), 128, 0, c->stream>>>(uwg_level_geom(c, 0), W, L.bc, mask_in, x, y);
    UWG_CUDA(c, cudaGetLastError());
    return UWG_OK;
}
template int uwg_q2_applyK<double>(uwg_ctx*, const double*, double*, bool);
template int uwg_q2_applyK<float>(uwg_ctx*, const float*, float*, bool);

int uwg_q2_diag(uwg_ctx* c, double* sinv) {
    if (c->dim == 3) return uwg_q2_3d_diag(c, sinv);
    const uwg_level& L = c->lev[0];
    k_diag_q2<<<nblk(L.n_el), 256, 0, c->stream>>>(uwg_level_geom(c, 0), L.W64, L.bc, L.diag64, sinv);
    UWG_CUDA(c, cudaGetLastError());
    return UWG_OK;
}

int uwg_q2_applyG(uwg_ctx* c, const double* p, double* y) {
    if (c->dim == 3) return uwg_q2_3d_applyG(c, p, y);
    vk_zero<double>(c->stream, c->n_vdof, y);
    k_applyG_q2<<<nblk(c->n_el), 256, 0, c->stream>>>(uwg_level_geom(c, 0), c->bc, p, y);
    UWG_CUDA(c, cudaGetLastError());
    return UWG_OK;
}

int uwg_q2_applyGt(uwg_ctx* c, const double* u, double* q, int only_bc) {
    if (c->dim == 3) return uwg_q2_3d_applyGt(c, u, q, only_bc);
    k_applyGt_q2<<<nblk(c->n_el), 256, 0, c->stream>>>(uwg_level_geom(c, 0), c->bc, only_bc, u, q);
    UWG_CUDA(c, cudaGetLastError());
    return UWG_OK;
}

int uwg_q2_schur_pc(uwg_ctx* c, const double* r, double* z) {
    if (c->dim == 3) return uwg_q2_3d_schur_pc(c, r, z);
    k_schur_pc_q2<<<nblk(c->n_el), 256, 0, c->stream>>>(c->n_el, c->Shat, r, z);
    UWG_CUDA(c, cudaGetLastError());
    return UWG_OK;
}

int uwg_q2_element_matrices(uwg_ctx* c, int64_t el, double* Ke, double* Ge, double* Se) {
    if (c->dim == 3) return uwg_q2_3d_element_matrices(c, el, Ke, Ge, Se);
    double* buf = nullptr;
    const int nk = 18 * 18, ng = 18 * 3, ns = 9;
    UWG_CUDA(c, cudaMallocAsync((void**)&buf, sizeof(double) * (nk + ng + ns), c->stream));
    k_element_matrices_q2<<<1, 1, 0, c->stream>>>(uwg_level_geom(c, 0), el, c->lev[0].W64, buf, buf + nk, buf + nk + ng);
    double h[18 * 18 + 18 * 3 + 9];
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaMemcpyAsync(h, buf, sizeof(h), cudaMemcpyDeviceToHost, c->stream);
    cudaFreeAsync(buf, c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) return uwg_set_error(c, UWG_ERR_CUDA, cudaGetErrorString(e));
    if (Ke) for (int i = 0; i < nk; i++) Ke[i] = h[i];
    if (Ge) for (int i = 0; i < ng; i++) Ge[i] = h[nk + i];
    if (Se) for (int i = 0; i < ns; i++) Se[i] = h[nk + ng + i];
    return UWG_OK;
}
