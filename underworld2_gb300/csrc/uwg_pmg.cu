// Multigrid for the pressure Laplacian L = G^T W G of the weighted BFBt Schur
// preconditioner on Q1/dQ0 meshes.
//
// Q1/dQ0 is not inf-sup stable: pressure fields of the form
// (-1)^(i+j+k) f(x) lie close to the kernel of G (exactly in it away from the
// walls when f depends on one coordinate only), so L has a whole branch of
// small eigenvalues on checkerboard-modulated smooth fields.  A multigrid with
// piecewise-constant coarse spaces cannot represent that branch and its CG
// iteration count grows with the mesh.  This hierarchy carries two unknowns
// per coarse cell from the first coarsening on: a smooth part and a
// checkerboard part, with prolongation
//     p_fine(i) = s(I) + (-1)^(i_x+i_y+i_z) c(I),      I = parent of i,
// and Galerkin coarse operators A_{l+1} = P^T A_l P.  Every level is stored as
// an explicit 3^dim-point cell stencil (2x2 blocks on coarse levels) in
// structure-of-arrays form, so an apply reads each coefficient once, coalesced.
//
// Layouts (n = cells of the level):
//   level 0  : st[o * n + e]                        = L[e, e + off(o)]
//   level >=1: st[((o * 2 + a) * 2 + b) * n + e]    = A[(a, e), (b, e + off(o))]
//   vectors  : level 0 x[e];  level >= 1 x[a * n + e]  (a = 0 smooth, 1 checkerboard)
//   off(o)   : o = (dx+1) + 3 (dy+1) + 9 (dz+1),  d* in {-1, 0, 1}
#include "uwg_ops.cuh"

namespace {

inline unsigned nblk(int64_t n, int t = 256) { return (unsigned)((n + t - 1) / t); }

template <int DIM>
__device__ __forceinline__ void cell_xyz(const uwg_lgeom& g, int64_t e, int& ex, int& ey, int& ez) {
    ex = (int)(e % g.res[0]);
    ey = (int)((e / g.res[0]) % g.res[1]);
    ez = DIM == 3 ? (int)(e / ((int64_t)g.res[0] * g.res[1])) : 0;
}

// |integral of dN/dx_d| over cell (ex, ey, ez) for each Q1 node (the sign
// is + for the node on the low side of axis d, - on the high side)
template <int DIM>
__device__ __forceinline__ void g_coef(const uwg_lgeom& g, int ex, int ey, int ez, float* a) {
    float hx = (float)(g.ax[0][ex + 1] - g.ax[0][ex]), hy = (float)(g.ax[1][ey + 1] - g.ax[1][ey]);
    float hz = DIM == 3 ? (float)(g.ax[2][ez + 1] - g.ax[2][ez]) : 2.0f;
    a[0] = 0.5f * hy * (DIM == 3 ? 0.5f * hz : 1.0f);
    a[1] = 0.5f * hx * (DIM == 3 ? 0.5f * hz : 1.0f);
    a[2] = 0.25f * hx * hy;
}

template <int DIM>
__device__ __forceinline__ bool in_grid(const uwg_lgeom& g, int x, int y, int z) {
    return x >= 0 && x < g.res[0] && y >= 0 && y < g.res[1] && (DIM == 2 || (z >= 0 && z < g.res[2]));
}

// Level-0 stencil of L = G^T W G; W is zero on Dirichlet dofs.
template <int DIM>
__global__ void k_pst0(uwg_lgeom g, const float* __restrict__ W, float* __restrict__ st) {
    constexpr int NO = DIM == 3 ? 27 : 9;
    int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (e >= g.n_el) return;
    int ex, ey, ez;
    cell_xyz<DIM>(g, e, ex, ey, ez);
    float a[3];
    g_coef<DIM>(g, ex, ey, ez, a);
    float acc[NO];
#pragma unroll
    for (int o = 0; o < NO; o++) acc[o] = 0.f;
#pragma unroll
    for (int ln = 0; ln < (1 << DIM); ln++) {
        const int lx = ln & 1, ly = (ln >> 1) & 1, lz = DIM == 3 ? (ln >> 2) & 1 : 0;
        int64_t node = (ex + lx) + (int64_t)g.nx[0] * ((ey + ly) + (int64_t)g.nx[1] * (ez + lz));
        float w[3] = {0.f, 0.f, 0.f};
#pragma unroll
        for (int d = 0; d < DIM; d++) w[d] = W[node * DIM + d];
        const float ge0 = lx ? -a[0] : a[0], ge1 = ly ? -a[1] : a[1], ge2 = lz ? -a[2] : a[2];
#pragma unroll
        for (int cn = 0; cn < (1 << DIM); cn++) {
            const int cx = cn & 1, cy = (cn >> 1) & 1, cz = DIM == 3 ? (cn >> 2) & 1 : 0;
            const int fx = ex + lx - 1 + cx, fy = ey + ly - 1 + cy, fz = DIM == 3 ? ez + lz - 1 + cz : 0;
            if (!in_grid<DIM>(g, fx, fy, fz)) continue;
            float b[3];
            g_coef<DIM>(g, fx, fy, fz, b);
            // the node is local corner (1-cx, 1-cy, 1-cz) of the neighbour
            float s = w[0] * ge0 * (cx ? b[0] : -b[0]) + w[1] * ge1 * (cy ? b[1] : -b[1]);
            if (DIM == 3) s += w[2] * ge2 * (cz ? b[2] : -b[2]);
            acc[(lx + cx) + 3 * (ly + cy) + (DIM == 3 ? 9 * (lz + cz) : 0)] += s;
        }
    }
#pragma unroll
    for (int o = 0; o < NO; o++) st[o * g.n_el + e] = acc[o];
}

// Coarse offset index of fine offset (o) seen from child (c) of a coarse cell:
// floor((c + o) / 2) per axis.
__host__ __device__ constexpr int coarse_off(int c, int o) { return ((c + o + 2) >> 1) - 1; }

// Galerkin level 0 (one unknown per cell) -> level 1 (smooth + checkerboard).
template <int DIM>
__global__ void k_pgal01(uwg_lgeom gf, uwg_lgeom gc, const float* __restrict__ st0, float* __restrict__ st1) {
    constexpr int NO = DIM == 3 ? 27 : 9;
    int64_t I = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (I >= gc.n_el) return;
    int X, Y, Z;
    cell_xyz<DIM>(gc, I, X, Y, Z);
    float acc[NO][4];
#pragma unroll
    for (int o = 0; o < NO; o++)
#pragma unroll
        for (int k = 0; k < 4; k++) acc[o][k] = 0.f;
    const int64_t nf = gf.n_el;
#pragma unroll
    for (int cn = 0; cn < (1 << DIM); cn++) {
        const int cx = cn & 1, cy = (cn >> 1) & 1, cz = DIM == 3 ? (cn >> 2) & 1 : 0;
        const int64_t i = (2 * X + cx) + (int64_t)gf.res[0] * ((2 * Y + cy) + (int64_t)gf.res[1] * (2 * Z + cz));
        const float si = ((cx + cy + cz) & 1) ? -1.f : 1.f;
#pragma unroll
        for (int o = 0; o < NO; o++) {
            const int ox = o % 3 - 1, oy = (o / 3) % 3 - 1, oz = DIM == 3 ? o / 9 - 1 : 0;
            const float v = st0[o * nf + i];
            const float sj = ((cx + ox + cy + oy + cz + oz) & 1) ? -1.f : 1.f;
            const int O = (coarse_off(cx, ox) + 1) + 3 * (coarse_off(cy, oy) + 1) +
                          (DIM == 3 ? 9 * (coarse_off(cz, oz) + 1) : 0);
            acc[O][0] += v;
            acc[O][1] += sj * v;
            acc[O][2] += si * v;
            acc[O][3] += si * sj * v;
        }
    }
#pragma unroll
    for (int o = 0; o < NO; o++)
#pragma unroll
        for (int k = 0; k < 4; k++) st1[(o * 4 + k) * gc.n_el + I] = acc[o][k];
}

// Galerkin level l -> l + 1, both with two unknowns per cell (aggregation per component).
template <int DIM>
__global__ void k_pgal22(uwg_lgeom gf, uwg_lgeom gc, const float* __restrict__ stf, float* __restrict__ stc) {
    constexpr int NO = DIM == 3 ? 27 : 9;
    int64_t I = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (I >= gc.n_el) return;
    int X, Y, Z;
    cell_xyz<DIM>(gc, I, X, Y, Z);
    float acc[NO][4];
#pragma unroll
    for (int o = 0; o < NO; o++)
#pragma unroll
        for (int k = 0; k < 4; k++) acc[o][k] = 0.f;
    const int64_t nf = gf.n_el;
#pragma unroll
    for (int cn = 0; cn < (1 << DIM); cn++) {
        const int cx = cn & 1, cy = (cn >> 1) & 1, cz = DIM == 3 ? (cn >> 2) & 1 : 0;
        const int64_t i = (2 * X + cx) + (int64_t)gf.res[0] * ((2 * Y + cy) + (int64_t)gf.res[1] * (2 * Z + cz));
#pragma unroll
        for (int o = 0; o < NO; o++) {
            const int ox = o % 3 - 1, oy = (o / 3) % 3 - 1, oz = DIM == 3 ? o / 9 - 1 : 0;
            const int O = (coarse_off(cx, ox) + 1) + 3 * (coarse_off(cy, oy) + 1) +
                          (DIM == 3 ? 9 * (coarse_off(cz, oz) + 1) : 0);
#pragma unroll
            for (int k = 0; k < 4; k++) acc[O][k] += stf[(o * 4 + k) * nf + i];
        }
    }
#pragma unroll
    for (int o = 0; o < NO; o++)
#pragma unroll
        for (int k = 0; k < 4; k++) stc[(o * 4 + k) * gc.n_el + I] = acc[o][k];
}

// y = A x on a level with nc unknowns per cell (1 or 2).  Branch-free: a
// neighbour outside the grid has a zero coefficient, so its index is only
// clamped into the array, and all loads of a thread can be in flight at once
// (the coarse levels are latency-bound otherwise).
template <int DIM, int NC>
__global__ void __launch_bounds__(256) k_papply(uwg_lgeom g, const float* __restrict__ st,
                                                const float* __restrict__ x, float* __restrict__ y) {
    constexpr int NO = DIM == 3 ? 27 : 9;
    constexpr int GRP = 9;   // offsets whose loads are issued together
    const int64_t n = g.n_el;
    int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (e >= n) return;
    const int64_t sy = g.res[0], sz = (int64_t)g.res[0] * g.res[1];
    float acc[NC];
#pragma unroll
    for (int a = 0; a < NC; a++) acc[a] = 0.f;
#pragma unroll
    for (int o0 = 0; o0 < NO; o0 += GRP) {
        float sv[GRP][NC * NC], xv[GRP][NC];
#pragma unroll
        for (int k = 0; k < GRP; k++) {
            const int o = o0 + k;
            const int ox = o % 3 - 1, oy = (o / 3) % 3 - 1, oz = DIM == 3 ? o / 9 - 1 : 0;
            int64_t j = e + ox + oy * sy + oz * sz;
            j = j < 0 ? 0 : (j >= n ? n - 1 : j);
#pragma unroll
            for (int q = 0; q < NC * NC; q++) sv[k][q] = __ldg(&st[(o * NC * NC + q) * n + e]);
#pragma unroll
            for (int b = 0; b < NC; b++) xv[k][b] = __ldg(&x[b * n + j]);
        }
#pragma unroll
        for (int k = 0; k < GRP; k++)
#pragma unroll
            for (int a = 0; a < NC; a++)
#pragma unroll
                for (int b = 0; b < NC; b++) acc[a] += sv[k][a * NC + b] * xv[k][b];
    }
#pragma unroll
    for (int a = 0; a < NC; a++) y[a * n + e] = acc[a];
}

template <int NC>
__global__ void k_pdiag(int64_t n, int center, const float* __restrict__ st, float* __restrict__ d) {
    int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (e >= n) return;
#pragma unroll
    for (int a = 0; a < NC; a++) {
        float v = st[(NC == 1 ? center : center * 4 + a * 3) * n + e];
        d[a * n + e] = v > 0.f ? v : 1.f;
    }
}

// rc = P^T rf between level lc-1 (ncf unknowns per cell) and lc (two per cell)
template <int DIM, int NCF>
__global__ void k_prestrict(uwg_lgeom gf, uwg_lgeom gc, const float* __restrict__ rf, float* __restrict__ rc) {
    int64_t I = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (I >= gc.n_el) return;
    int X, Y, Z;
    cell_xyz<DIM>(gc, I, X, Y, Z);
    float s0 = 0.f, s1 = 0.f;
#pragma unroll
    for (int cn = 0; cn < (1 << DIM); cn++) {
        const int cx = cn & 1, cy = (cn >> 1) & 1, cz = DIM == 3 ? (cn >> 2) & 1 : 0;
        const int64_t i = (2 * X + cx) + (int64_t)gf.res[0] * ((2 * Y + cy) + (int64_t)gf.res[1] * (2 * Z + cz));
        if constexpr (NCF == 1) {
            const float v = rf[i];
            s0 += v;
            s1 += ((cx + cy + cz) & 1) ? -v : v;
        } else {
            s0 += rf[i];
            s1 += rf[gf.n_el + i];
        }
    }
    rc[I] = s0;
    rc[gc.n_el + I] = s1;
}

// xf += P xc
template <int DIM, int NCF>
__global__ void k_pprolong_add(uwg_lgeom gf, uwg_lgeom gc, const float* __restrict__ xc, float* __restrict__ xf) {
    int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= gf.n_el) return;
    int x, y, z;
    cell_xyz<DIM>(gf, i, x, y, z);
    const int64_t I = (x >> 1) + (int64_t)gc.res[0] * ((y >> 1) + (int64_t)gc.res[1] * (z >> 1));
    if constexpr (NCF == 1) {
        const float c = xc[gc.n_el + I];
        xf[i] += xc[I] + (((x + y + z) & 1) ? -c : c);
    } else {
        xf[i] += xc[I];
        xf[gf.n_el + i] += xc[gc.n_el + I];
    }
}

// Dense (ncomp n) x (ncomp n) matrix of a level, FP64, plus tau/n on the
// smooth-smooth block: the constant pressure is the kernel of L, and adding
// tau v v^T (v the normalised constant) makes the matrix invertible without
// changing its action on the complement of v.
template <int DIM, int NC>
__global__ void k_pdense(uwg_lgeom g, const float* __restrict__ st, double* __restrict__ A) {
    constexpr int NO = DIM == 3 ? 27 : 9;
    const int64_t n = g.n_el, m = NC * n;
    int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (e >= n) return;
    int ex, ey, ez;
    cell_xyz<DIM>(g, e, ex, ey, ez);
    for (int o = 0; o < NO; o++) {
        const int ox = o % 3 - 1, oy = (o / 3) % 3 - 1, oz = DIM == 3 ? o / 9 - 1 : 0;
        if (!in_grid<DIM>(g, ex + ox, ey + oy, ez + oz)) continue;
        const int64_t j = e + ox + (int64_t)oy * g.res[0] + (int64_t)oz * g.res[0] * g.res[1];
        for (int a = 0; a < NC; a++)
            for (int b = 0; b < NC; b++)
                A[(a * n + e) * m + b * n + j] = st[(NC == 1 ? o : o * 4 + a * 2 + b) * n + e];
    }
}

// Rank-one terms tau 1 1^T on the smooth block (and, when the checkerboard is a
// null mode of G as well, on the checkerboard block) make the singular coarse
// operator invertible without changing its action on the range.  A one-unknown
// level (m == n) gets the checkerboard term as tau s s^T, s_i = (-1)^(x+y+z).
__global__ void k_pdense_fix(int64_t m, int64_t n, int fix_checkerboard, int rx, int ry, double* A) {
    __shared__ double red[1024];
    if (fix_checkerboard && m == n) {
        double mx = 0.0;
        for (int64_t i = threadIdx.x; i < n; i += blockDim.x) mx = fmax(mx, A[i * m + i]);
        red[threadIdx.x] = mx;
        __syncthreads();
        for (int s = blockDim.x / 2; s > 0; s >>= 1) {
            if ((int)threadIdx.x < s) red[threadIdx.x] = fmax(red[threadIdx.x], red[threadIdx.x + s]);
            __syncthreads();
        }
        const double tau = (red[0] > 0.0 ? red[0] : 1.0) / (double)n;
        __syncthreads();
        for (int64_t k = threadIdx.x; k < n * n; k += blockDim.x) {
            const int64_t i = k / n, j = k % n;
            const int si = (int)((i % rx) + (i / rx) % ry + i / ((int64_t)rx * ry)) & 1;
            const int sj = (int)((j % rx) + (j / rx) % ry + j / ((int64_t)rx * ry)) & 1;
            A[i * m + j] += si == sj ? tau : -tau;
        }
        __syncthreads();
    }
    for (int blk = 0; blk < (fix_checkerboard && m == 2 * n ? 2 : 1); blk++) {
        double* B = A + (int64_t)blk * n * m + (int64_t)blk * n;   // diagonal block blk
        double mx = 0.0;
        for (int64_t i = threadIdx.x; i < n; i += blockDim.x) mx = fmax(mx, B[i * m + i]);
        red[threadIdx.x] = mx;
        __syncthreads();
        for (int s = blockDim.x / 2; s > 0; s >>= 1) {
            if ((int)threadIdx.x < s) red[threadIdx.x] = fmax(red[threadIdx.x], red[threadIdx.x + s]);
            __syncthreads();
        }
        const double tau = (red[0] > 0.0 ? red[0] : 1.0) / (double)n;
        __syncthreads();
        for (int64_t k = threadIdx.x; k < n * n; k += blockDim.x) B[(k / n) * m + (k % n)] += tau;
        __syncthreads();
    }
}


// Level-0 apply without the stencil (3D): y = G^T (W (G x)).  A CTA owns a
// 16x8x8 tile of cells; it stages the tile's cell values with a one-cell halo
// in shared memory, forms W G x at the tile's 17x9x9 nodes in shared memory,
// and then sums G^T over each cell's eight nodes.  DRAM traffic is x, W (three
// floats per node) and y: about a sixth of the 27-coefficient stencil's.  The
// tile's W is copied into shared memory with cp.async first, so its latency
// overlaps the staging of x.
__device__ __forceinline__ void pmg_cp_async4(void* smem, const void* gmem) {
    unsigned sa = (unsigned)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(sa), "l"(gmem));
}
// as pmg_cp_async4, writing zero instead when `valid` is false (src-size 0)
__device__ __forceinline__ void pmg_cp_async4z(void* smem, const void* gmem, bool valid) {
    unsigned sa = (unsigned)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4, %2;\n" ::"r"(sa), "l"(gmem), "r"(valid ? 4 : 0));
}
#define PT_X 16
#define PT_Y 8
#define PT_Z 8
// cell size along axis d of halo cell i of a tile starting at t0 (0 outside the grid)
__device__ __forceinline__ float pmg_hcell(const uwg_lgeom& g, int d, int t0, int i) {
    const int c0 = t0 - 1 + i;
    const int r = d == 0 ? g.res[0] : d == 1 ? g.res[1] : g.res[2];
    const double* a = d == 0 ? g.ax[0] : d == 1 ? g.ax[1] : g.ax[2];
    return (c0 >= 0 && c0 < r) ? (float)(a[c0 + 1] - a[c0]) : 0.f;
}

__global__ void __launch_bounds__(256) k_papply0_mf(uwg_lgeom g, const float* __restrict__ W,
                                                    const float* __restrict__ x, float* __restrict__ y) {
    constexpr int HX = PT_X + 2, HY = PT_Y + 2, HZ = PT_Z + 2, NH = HX * HY * HZ, HXY = HX * HY;
    constexpr int NX = PT_X + 1, NY = PT_Y + 1, NZ = PT_Z + 1, NN = NX * NY * NZ, NXY = NX * NY;
    __shared__ float ps[NH];
    __shared__ float vs[3][NN];
    // face areas of the halo cells, / 4: A0 = hy hz, A1 = hx hz, A2 = hx hy
    __shared__ float A0[HY][HZ], A1[HX][HZ], A2[HX][HY];
    const int ntx = (g.res[0] + PT_X - 1) / PT_X, nty = (g.res[1] + PT_Y - 1) / PT_Y;
    const int tile = blockIdx.x;
    const int tx0 = (tile % ntx) * PT_X, ty0 = ((tile / ntx) % nty) * PT_Y, tz0 = (tile / (ntx * nty)) * PT_Z;
    const int64_t sy = g.res[0], sz = (int64_t)g.res[0] * g.res[1];
    for (int k = threadIdx.x; k < NN; k += blockDim.x) {
        const int ni = k % NX, nj = (k / NX) % NY, nk = k / NXY;
        const int gi = tx0 + ni, gj = ty0 + nj, gk = tz0 + nk;
        if (gi < g.nx[0] && gj < g.nx[1] && gk < g.nx[2]) {
            const float* src = W + (gi + (int64_t)g.nx[0] * (gj + (int64_t)g.nx[1] * gk)) * 3;
            pmg_cp_async4(&vs[0][k], src);
            pmg_cp_async4(&vs[1][k], src + 1);
            pmg_cp_async4(&vs[2][k], src + 2);
        }
    }
    for (int k = threadIdx.x; k < NH; k += blockDim.x) {
        const int i = k % HX, j = (k / HX) % HY, l = k / HXY;
        const int cx = tx0 - 1 + i, cy = ty0 - 1 + j, cz = tz0 - 1 + l;
        const bool in = in_grid<3>(g, cx, cy, cz);
        pmg_cp_async4z(&ps[k], x + (in ? cx + sy * cy + sz * cz : 0), in);
    }
    for (int t = threadIdx.x; t < HY * HZ + HX * HZ + HX * HY; t += blockDim.x) {
        if (t < HY * HZ) {
            const int j = t / HZ, l = t % HZ;
            A0[j][l] = 0.25f * pmg_hcell(g, 1, ty0, j) * pmg_hcell(g, 2, tz0, l);
        } else if (t < HY * HZ + HX * HZ) {
            const int u = t - HY * HZ, i = u / HZ, l = u % HZ;
            A1[i][l] = 0.25f * pmg_hcell(g, 0, tx0, i) * pmg_hcell(g, 2, tz0, l);
        } else {
            const int u = t - HY * HZ - HX * HZ, i = u / HY, j = u % HY;
            A2[i][j] = 0.25f * pmg_hcell(g, 0, tx0, i) * pmg_hcell(g, 1, ty0, j);
        }
    }
    asm volatile("cp.async.commit_group;\n\tcp.async.wait_group 0;\n" ::: "memory");
    __syncthreads();
    // W G x at the tile's nodes: differences of the eight surrounding cells
    for (int k = threadIdx.x; k < NN; k += blockDim.x) {
        const int ni = k % NX, nj = (k / NX) % NY, nk = k / NXY;
        const int gi = tx0 + ni, gj = ty0 + nj, gk = tz0 + nk;
        float v0 = 0.f, v1 = 0.f, v2 = 0.f;
        if (gi < g.nx[0] && gj < g.nx[1] && gk < g.nx[2]) {
            const float* P = &ps[ni + HX * nj + HXY * nk];
            const float p000 = P[0], p100 = P[1], p010 = P[HX], p110 = P[HX + 1];
            const float p001 = P[HXY], p101 = P[HXY + 1], p011 = P[HXY + HX], p111 = P[HXY + HX + 1];
            v0 = A0[nj][nk] * (p100 - p000) + A0[nj + 1][nk] * (p110 - p010) + A0[nj][nk + 1] * (p101 - p001) +
                 A0[nj + 1][nk + 1] * (p111 - p011);
            v1 = A1[ni][nk] * (p010 - p000) + A1[ni + 1][nk] * (p110 - p100) + A1[ni][nk + 1] * (p011 - p001) +
                 A1[ni + 1][nk + 1] * (p111 - p101);
            v2 = A2[ni][nj] * (p001 - p000) + A2[ni + 1][nj] * (p101 - p100) + A2[ni][nj + 1] * (p011 - p010) +
                 A2[ni + 1][nj + 1] * (p111 - p110);
            v0 *= vs[0][k];
            v1 *= vs[1][k];
            v2 *= vs[2][k];
        }
        vs[0][k] = v0;
        vs[1][k] = v1;
        vs[2][k] = v2;
    }
    __syncthreads();
    // G^T: each cell sums its eight nodes, grouped by face
    for (int k = threadIdx.x; k < PT_X * PT_Y * PT_Z; k += blockDim.x) {
        const int i = k % PT_X, j = (k / PT_X) % PT_Y, l = k / (PT_X * PT_Y);
        const int ex = tx0 + i, ey = ty0 + j, ez = tz0 + l;
        if (!in_grid<3>(g, ex, ey, ez)) continue;
        const int q = i + NX * j + NXY * l;
        const float* V0 = &vs[0][q];
        const float* V1 = &vs[1][q];
        const float* V2 = &vs[2][q];
        const float d0 = (V0[0] - V0[1]) + (V0[NX] - V0[NX + 1]) + (V0[NXY] - V0[NXY + 1]) + (V0[NXY + NX] - V0[NXY + NX + 1]);
        const float d1 = (V1[0] - V1[NX]) + (V1[1] - V1[NX + 1]) + (V1[NXY] - V1[NXY + NX]) + (V1[NXY + 1] - V1[NXY + NX + 1]);
        const float d2 = (V2[0] - V2[NXY]) + (V2[1] - V2[NXY + 1]) + (V2[NX] - V2[NXY + NX]) + (V2[NX + 1] - V2[NXY + NX + 1]);
        y[ex + sy * ey + sz * ez] = A0[j + 1][l + 1] * d0 + A1[i + 1][l + 1] * d1 + A2[i + 1][j + 1] * d2;
    }
}

// ---------------------------------------------------------------------------
// Smooth checkerboard coarse space on the first coarsening.  With piecewise-
// constant interpolation of the checkerboard component the CG iteration count
// of L still grows with the mesh (the checkerboard branch of L behaves like a
// fourth-order operator); interpolating that component cell-centred
// trilinearly instead,
//     p_fine(i) += (-1)^(i_x+i_y+i_z) sum_J w(i, J) c(J)
// (weights 3/4, 1/4 per axis, clipped onto the cell itself at the walls),
// halves it on 32^3 and more on finer meshes.  Level 1 then carries a
// 5^dim-point checkerboard-checkerboard block, stored after the 3^dim x 2 x 2
// blocks; deeper levels aggregate piecewise-constantly again, which brings
// the stencil back to 3^dim points.
// ---------------------------------------------------------------------------
// 1D trilinear support of fine cell f: (p, 3/4) and (q, 1/4), q clipped to p at the walls
__device__ __forceinline__ void tri1d(int f, int rc, int& p, int& q) {
    p = f >> 1;
    q = (f & 1) ? p + 1 : p - 1;
    if (q < 0 || q >= rc) q = p;
}
// weight of coarse cell I in fine cell f's 1D support
__device__ __forceinline__ float tri1w(int f, int rc, int I) {
    int p, q;
    tri1d(f, rc, p, q);
    return (p == I ? 0.75f : 0.f) + (q == I ? 0.25f : 0.f);
}

template <int DIM>
__global__ void __launch_bounds__(128) k_pgal01_tri(uwg_lgeom gf, uwg_lgeom gc, const float* __restrict__ st0,
                                                    float* __restrict__ st1, float* __restrict__ cc5) {
    constexpr int NO = DIM == 3 ? 27 : 9, N5 = DIM == 3 ? 125 : 25, NF = DIM == 3 ? 64 : 16;
    __shared__ float ss[NO], sc[NO], cs[NO], cc[N5];
    const int64_t I = blockIdx.x;
    const int64_t nf = gf.n_el, nc = gc.n_el;
    int X, Y, Z;
    cell_xyz<DIM>(gc, I, X, Y, Z);
    const int rc[3] = {gc.res[0], gc.res[1], DIM == 3 ? gc.res[2] : 1};
    for (int k = threadIdx.x; k < N5; k += blockDim.x) {
        cc[k] = 0.f;
        if (k < NO) { ss[k] = 0.f; sc[k] = 0.f; cs[k] = 0.f; }
    }
    __syncthreads();
    // rows of the smooth component: the children of I (weight 1)
    for (int t = threadIdx.x; t < (1 << DIM) * NO; t += blockDim.x) {
        const int ch = t / NO, o = t % NO;
        const int ix = 2 * X + (ch & 1), iy = 2 * Y + ((ch >> 1) & 1), iz = DIM == 3 ? 2 * Z + (ch >> 2) : 0;
        const int64_t i = ix + (int64_t)gf.res[0] * (iy + (int64_t)gf.res[1] * iz);
        const float v = st0[o * nf + i];
        if (v == 0.f) continue;
        const int jx = ix + o % 3 - 1, jy = iy + (o / 3) % 3 - 1, jz = DIM == 3 ? iz + o / 9 - 1 : 0;
        if (!in_grid<DIM>(gf, jx, jy, jz)) continue;
        atomicAdd(&ss[((jx >> 1) - X + 1) + 3 * ((jy >> 1) - Y + 1) + (DIM == 3 ? 9 * ((jz >> 1) - Z + 1) : 0)], v);
        const float vj = ((jx + jy + jz) & 1) ? -v : v;
        int px, qx, py, qy, pz = 0, qz = 0;
        tri1d(jx, rc[0], px, qx);
        tri1d(jy, rc[1], py, qy);
        if (DIM == 3) tri1d(jz, rc[2], pz, qz);
        for (int cz = 0; cz < (DIM == 3 ? 2 : 1); cz++)
            for (int cy = 0; cy < 2; cy++)
                for (int cx = 0; cx < 2; cx++) {
                    const int Jx = cx ? qx : px, Jy = cy ? qy : py, Jz = cz ? qz : pz;
                    const float w = (cx ? 0.25f : 0.75f) * (cy ? 0.25f : 0.75f) * (DIM == 3 ? (cz ? 0.25f : 0.75f) : 1.f);
                    atomicAdd(&sc[(Jx - X + 1) + 3 * (Jy - Y + 1) + (DIM == 3 ? 9 * (Jz - Z + 1) : 0)], w * vj);
                }
    }
    // rows of the checkerboard component: the fine cells of I's trilinear support
    for (int t = threadIdx.x; t < NF * NO; t += blockDim.x) {
        const int f = t / NO, o = t % NO;
        const int ix = 2 * X - 1 + (f & 3), iy = 2 * Y - 1 + ((f >> 2) & 3), iz = DIM == 3 ? 2 * Z - 1 + (f >> 4) : 0;
        if (!in_grid<DIM>(gf, ix, iy, iz)) continue;
        const float wi = tri1w(ix, rc[0], X) * tri1w(iy, rc[1], Y) * (DIM == 3 ? tri1w(iz, rc[2], Z) : 1.f);
        if (wi == 0.f) continue;
        const int64_t i = ix + (int64_t)gf.res[0] * (iy + (int64_t)gf.res[1] * iz);
        const float v0 = st0[o * nf + i];
        if (v0 == 0.f) continue;
        const float v = (((ix + iy + iz) & 1) ? -wi : wi) * v0;
        const int jx = ix + o % 3 - 1, jy = iy + (o / 3) % 3 - 1, jz = DIM == 3 ? iz + o / 9 - 1 : 0;
        if (!in_grid<DIM>(gf, jx, jy, jz)) continue;
        atomicAdd(&cs[((jx >> 1) - X + 1) + 3 * ((jy >> 1) - Y + 1) + (DIM == 3 ? 9 * ((jz >> 1) - Z + 1) : 0)], v);
        const float vj = ((jx + jy + jz) & 1) ? -v : v;
        int px, qx, py, qy, pz = 0, qz = 0;
        tri1d(jx, rc[0], px, qx);
        tri1d(jy, rc[1], py, qy);
        if (DIM == 3) tri1d(jz, rc[2], pz, qz);
        for (int cz = 0; cz < (DIM == 3 ? 2 : 1); cz++)
            for (int cy = 0; cy < 2; cy++)
                for (int cx = 0; cx < 2; cx++) {
                    const int Jx = cx ? qx : px, Jy = cy ? qy : py, Jz = cz ? qz : pz;
                    const float w = (cx ? 0.25f : 0.75f) * (cy ? 0.25f : 0.75f) * (DIM == 3 ? (cz ? 0.25f : 0.75f) : 1.f);
                    atomicAdd(&cc[(Jx - X + 2) + 5 * (Jy - Y + 2) + (DIM == 3 ? 25 * (Jz - Z + 2) : 0)], w * vj);
                }
    }
    __syncthreads();
    for (int k = threadIdx.x; k < N5; k += blockDim.x) {
        cc5[k * nc + I] = cc[k];
        if (k < NO) {
            st1[(k * 4 + 0) * nc + I] = ss[k];
            st1[(k * 4 + 1) * nc + I] = sc[k];
            st1[(k * 4 + 2) * nc + I] = cs[k];
            st1[(k * 4 + 3) * nc + I] = 0.f;
        }
    }
}

// Galerkin level 1 (smooth checkerboard block) -> level 2 (piecewise constant)
template <int DIM>
__global__ void k_pgal12(uwg_lgeom gf, uwg_lgeom gc, const float* __restrict__ stf, const float* __restrict__ cc5,
                         float* __restrict__ stc) {
    constexpr int NO = DIM == 3 ? 27 : 9, N5 = DIM == 3 ? 125 : 25;
    int64_t I = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (I >= gc.n_el) return;
    int X, Y, Z;
    cell_xyz<DIM>(gc, I, X, Y, Z);
    float acc[NO][4];
#pragma unroll
    for (int o = 0; o < NO; o++)
#pragma unroll
        for (int k = 0; k < 4; k++) acc[o][k] = 0.f;
    const int64_t nf = gf.n_el;
    for (int cn = 0; cn < (1 << DIM); cn++) {
        const int cx = cn & 1, cy = (cn >> 1) & 1, cz = DIM == 3 ? (cn >> 2) & 1 : 0;
        const int64_t i = (2 * X + cx) + (int64_t)gf.res[0] * ((2 * Y + cy) + (int64_t)gf.res[1] * (2 * Z + cz));
#pragma unroll
        for (int o = 0; o < NO; o++) {
            const int ox = o % 3 - 1, oy = (o / 3) % 3 - 1, oz = DIM == 3 ? o / 9 - 1 : 0;
            const int O = (coarse_off(cx, ox) + 1) + 3 * (coarse_off(cy, oy) + 1) +
                          (DIM == 3 ? 9 * (coarse_off(cz, oz) + 1) : 0);
#pragma unroll
            for (int k = 0; k < 3; k++) acc[O][k] += stf[(o * 4 + k) * nf + i];
        }
#pragma unroll
        for (int o = 0; o < N5; o++) {
            const int ox = o % 5 - 2, oy = (o / 5) % 5 - 2, oz = DIM == 3 ? o / 25 - 2 : 0;
            const int O = (((cx + ox + 4) >> 1) - 1) + 3 * (((cy + oy + 4) >> 1) - 1) +
                          (DIM == 3 ? 9 * (((cz + oz + 4) >> 1) - 1) : 0);
            acc[O][3] += cc5[o * nf + i];
        }
    }
#pragma unroll
    for (int o = 0; o < NO; o++)
#pragma unroll
        for (int k = 0; k < 4; k++) stc[(o * 4 + k) * gc.n_el + I] = acc[o][k];
}

// y = A_1 x on level 1 with the smooth checkerboard block (branch-free, clamped)
template <int DIM>
__global__ void __launch_bounds__(256) k_papply1_tri(uwg_lgeom g, const float* __restrict__ st,
                                                     const float* __restrict__ cc5, const float* __restrict__ x,
                                                     float* __restrict__ y) {
    constexpr int NO = DIM == 3 ? 27 : 9, N5 = DIM == 3 ? 125 : 25;
    const int64_t n = g.n_el;
    int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (e >= n) return;
    const int64_t sy = g.res[0], sz = (int64_t)g.res[0] * g.res[1];
    float a0 = 0.f, a1 = 0.f;
#pragma unroll 9
    for (int o = 0; o < NO; o++) {
        const int ox = o % 3 - 1, oy = (o / 3) % 3 - 1, oz = DIM == 3 ? o / 9 - 1 : 0;
        int64_t j = e + ox + oy * sy + oz * sz;
        j = j < 0 ? 0 : (j >= n ? n - 1 : j);
        const float xs = __ldg(&x[j]), xc = __ldg(&x[n + j]);
        a0 += __ldg(&st[(o * 4 + 0) * n + e]) * xs + __ldg(&st[(o * 4 + 1) * n + e]) * xc;
        a1 += __ldg(&st[(o * 4 + 2) * n + e]) * xs;
    }
#pragma unroll 25
    for (int o = 0; o < N5; o++) {
        const int ox = o % 5 - 2, oy = (o / 5) % 5 - 2, oz = DIM == 3 ? o / 25 - 2 : 0;
        int64_t j = e + ox + oy * sy + oz * sz;
        j = j < 0 ? 0 : (j >= n ? n - 1 : j);
        a1 += __ldg(&cc5[o * n + e]) * __ldg(&x[n + j]);
    }
    y[e] = a0;
    y[n + e] = a1;
}

// rc = P^T rf, level 0 -> 1, smooth checkerboard component.  The 1D weights of
// the four fine cells 2X-1 .. 2X+2 are formed once per axis.
template <int DIM>
__global__ void k_prestrict_tri(uwg_lgeom gf, uwg_lgeom gc, const float* __restrict__ rf, float* __restrict__ rc_) {
    int64_t I = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (I >= gc.n_el) return;
    int X[3];
    cell_xyz<DIM>(gc, I, X[0], X[1], X[2]);
    float w[3][4];
    int lo[3], hi[3];
#pragma unroll
    for (int d = 0; d < 3; d++) {
        const int rf_d = d == 0 ? gf.res[0] : d == 1 ? gf.res[1] : gf.res[2];
        const int rc_d = d == 0 ? gc.res[0] : d == 1 ? gc.res[1] : gc.res[2];
        lo[d] = 0;
        hi[d] = (d < DIM) ? 4 : 1;
#pragma unroll
        for (int k = 0; k < 4; k++) {
            const int f = 2 * X[d] - 1 + k;
            w[d][k] = (d < DIM && f >= 0 && f < rf_d) ? tri1w(f, rc_d, X[d]) : 0.f;
        }
        if (d >= DIM) w[d][0] = 1.f;
    }
    const int64_t sy = gf.res[0], sz = (int64_t)gf.res[0] * gf.res[1];
    float s0 = 0.f, s1 = 0.f;
    for (int c = lo[2]; c < hi[2]; c++) {
        const int iz = DIM == 3 ? 2 * X[2] - 1 + c : 0;
        if (DIM == 3 && (iz < 0 || iz >= gf.res[2])) continue;
        for (int b = 0; b < 4; b++) {
            const int iy = 2 * X[1] - 1 + b;
            if (iy < 0 || iy >= gf.res[1]) continue;
            const float wyz = w[1][b] * w[2][c];
            const float* row = rf + iy * sy + iz * sz;
            const bool child_yz = (b == 1 || b == 2) && (DIM == 2 || c == 1 || c == 2);
#pragma unroll
            for (int a = 0; a < 4; a++) {
                const int ix = 2 * X[0] - 1 + a;
                if (ix < 0 || ix >= gf.res[0]) continue;
                const float v = row[ix];
                if (child_yz && (a == 1 || a == 2)) s0 += v;
                const float wv = w[0][a] * wyz * v;
                s1 += ((ix + iy + iz) & 1) ? -wv : wv;
            }
        }
    }
    rc_[I] = s0;
    rc_[gc.n_el + I] = s1;
}

// xf += P xc, level 1 -> 0, smooth checkerboard component
template <int DIM>
__global__ void k_pprolong_tri(uwg_lgeom gf, uwg_lgeom gc, const float* __restrict__ xc, float* __restrict__ xf) {
    int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= gf.n_el) return;
    int x, y, z;
    cell_xyz<DIM>(gf, i, x, y, z);
    const int64_t nc = gc.n_el, sy = gc.res[0], sz = (int64_t)gc.res[0] * gc.res[1];
    int px, qx, py, qy, pz = 0, qz = 0;
    tri1d(x, gc.res[0], px, qx);
    tri1d(y, gc.res[1], py, qy);
    if (DIM == 3) tri1d(z, gc.res[2], pz, qz);
    float c = 0.f;
#pragma unroll
    for (int cz = 0; cz < (DIM == 3 ? 2 : 1); cz++)
#pragma unroll
        for (int cy = 0; cy < 2; cy++)
#pragma unroll
            for (int cx = 0; cx < 2; cx++) {
                const float w = (cx ? 0.25f : 0.75f) * (cy ? 0.25f : 0.75f) * (DIM == 3 ? (cz ? 0.25f : 0.75f) : 1.f);
                c += w * xc[nc + (cx ? qx : px) + sy * (cy ? qy : py) + sz * (cz ? qz : pz)];
            }
    xf[i] += xc[(x >> 1) + sy * (y >> 1) + sz * (DIM == 3 ? (z >> 1) : 0)] + (((x + y + z) & 1) ? -c : c);
}

__global__ void k_pdiag1_tri(int64_t n, int center, int center5, const float* __restrict__ st,
                             const float* __restrict__ cc5, float* __restrict__ d) {
    int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (e >= n) return;
    const float a = st[(center * 4) * n + e], b = cc5[center5 * n + e];
    d[e] = a > 0.f ? a : 1.f;
    d[n + e] = b > 0.f ? b : 1.f;
}
}  // namespace

#define PMG_DIM(KERN, GRID, ...)                                               \
    do {                                                                        \
        if (c->dim == 3) KERN<3><<<GRID, 256, 0, c->stream>>>(__VA_ARGS__);    \
        else KERN<2><<<GRID, 256, 0, c->stream>>>(__VA_ARGS__);                \
    } while (0)
#define PMG_DIM_NC(KERN, NC, GRID, ...)                                                        \
    do {                                                                                        \
        if (c->dim == 3) {                                                                      \
            if (NC == 1) KERN<3, 1><<<GRID, 256, 0, c->stream>>>(__VA_ARGS__);                 \
            else KERN<3, 2><<<GRID, 256, 0, c->stream>>>(__VA_ARGS__);                         \
        } else {                                                                                \
            if (NC == 1) KERN<2, 1><<<GRID, 256, 0, c->stream>>>(__VA_ARGS__);                 \
            else KERN<2, 2><<<GRID, 256, 0, c->stream>>>(__VA_ARGS__);                         \
        }                                                                                       \
    } while (0)

int uwg_pmg_ncomp(int l) { return l == 0 ? 1 : 2; }

// level 1 uses the smooth checkerboard interpolation when it is not the coarsest level
static bool smooth1(const uwg_ctx* c) { return c->pnlev >= 3; }

int64_t uwg_pmg_stencil_size(const uwg_ctx* c, int l) {
    int no = c->dim == 3 ? 27 : 9, n5 = c->dim == 3 ? 125 : 25;
    int64_t s = (int64_t)no * (l == 0 ? 1 : 4) * c->lev[l].n_el;
    if (l == 1 && smooth1(c)) s += (int64_t)n5 * c->lev[l].n_el;   // 5^dim checkerboard block after the 3^dim blocks
    return s;
}
static float* cc5_of(const uwg_ctx* c, const float* st1) {
    return (float*)st1 + (int64_t)(c->dim == 3 ? 27 : 9) * 4 * c->lev[1].n_el;
}

int uwg_pmg_stencil(uwg_ctx* c, int l, const float* W0, const float* st_fine, float* st) {
    if (l == 0) {
        uwg_lgeom g = uwg_level_geom(c, 0);
        PMG_DIM(k_pst0, nblk(g.n_el), g, W0, st);
    } else {
        uwg_lgeom gf = uwg_level_geom(c, l - 1), gc = uwg_level_geom(c, l);
        if (l == 1 && smooth1(c)) {
            if (c->dim == 3) k_pgal01_tri<3><<<(unsigned)gc.n_el, 128, 0, c->stream>>>(gf, gc, st_fine, st, cc5_of(c, st));
            else k_pgal01_tri<2><<<(unsigned)gc.n_el, 128, 0, c->stream>>>(gf, gc, st_fine, st, cc5_of(c, st));
        } else if (l == 1) {
            PMG_DIM(k_pgal01, nblk(gc.n_el, 128), gf, gc, st_fine, st);
        } else if (l == 2 && smooth1(c)) {
            PMG_DIM(k_pgal12, nblk(gc.n_el, 128), gf, gc, st_fine, cc5_of(c, st_fine), st);
        } else {
            PMG_DIM(k_pgal22, nblk(gc.n_el, 128), gf, gc, st_fine, st);
        }
    }
    UWG_CUDA(c, cudaGetLastError());
    return UWG_OK;
}

int uwg_pmg_apply(uwg_ctx* c, int l, const float* st, const float* x, float* y) {
    uwg_lgeom g = uwg_level_geom(c, l);
    if (l == 1 && smooth1(c)) {
        PMG_DIM(k_papply1_tri, nblk(g.n_el), g, st, cc5_of(c, st), x, y);
        UWG_CUDA(c, cudaGetLastError());
        return UWG_OK;
    }
    PMG_DIM_NC(k_papply, uwg_pmg_ncomp(l), nblk(g.n_el), g, st, x, y);
    UWG_CUDA(c, cudaGetLastError());
    return UWG_OK;
}

int uwg_pmg_apply0_mf(uwg_ctx* c, const float* W0, const float* x, float* y) {
    if (c->dim != 3) return uwg_set_error(c, UWG_ERR_ARG, "matrix-free pressure apply is 3D only");
    const uwg_level& L = c->lev[0];
    unsigned tiles = (unsigned)(((L.res[0] + PT_X - 1) / PT_X) * ((L.res[1] + PT_Y - 1) / PT_Y) *
                                ((L.res[2] + PT_Z - 1) / PT_Z));
    k_papply0_mf<<<tiles, 256, 0, c->stream>>>(uwg_level_geom(c, 0), W0, x, y);
    UWG_CUDA(c, cudaGetLastError());
    return UWG_OK;
}

int uwg_pmg_diag(uwg_ctx* c, int l, const float* st, float* d) {
    int64_t n = c->lev[l].n_el;
    int center = c->dim == 3 ? 13 : 4;
    if (l == 0) k_pdiag<1><<<nblk(n), 256, 0, c->stream>>>(n, center, st, d);
    else if (l == 1 && smooth1(c)) k_pdiag1_tri<<<nblk(n), 256, 0, c->stream>>>(n, center, c->dim == 3 ? 62 : 12, st, cc5_of(c, st), d);
    else k_pdiag<2><<<nblk(n), 256, 0, c->stream>>>(n, center, st, d);
    UWG_CUDA(c, cudaGetLastError());
    return UWG_OK;
}

int uwg_pmg_restrict(uwg_ctx* c, int lc, const float* rf, float* rc) {
    uwg_lgeom gf = uwg_level_geom(c, lc - 1), gc = uwg_level_geom(c, lc);
    if (lc == 1 && smooth1(c)) PMG_DIM(k_prestrict_tri, nblk(gc.n_el), gf, gc, rf, rc);
    else PMG_DIM_NC(k_prestrict, uwg_pmg_ncomp(lc - 1), nblk(gc.n_el), gf, gc, rf, rc);
    UWG_CUDA(c, cudaGetLastError());
    return UWG_OK;
}

int uwg_pmg_prolong_add(uwg_ctx* c, int lc, const float* xc, float* xf) {
    uwg_lgeom gf = uwg_level_geom(c, lc - 1), gc = uwg_level_geom(c, lc);
    if (lc == 1 && smooth1(c)) PMG_DIM(k_pprolong_tri, nblk(gf.n_el), gf, gc, xc, xf);
    else PMG_DIM_NC(k_pprolong_add, uwg_pmg_ncomp(lc - 1), nblk(gf.n_el), gf, gc, xc, xf);
    UWG_CUDA(c, cudaGetLastError());
    return UWG_OK;
}

int uwg_pmg_dense_inverse(uwg_ctx* c, int l, const float* st, int fix_checkerboard, float* inv32) {
    uwg_lgeom g = uwg_level_geom(c, l);
    int nc = uwg_pmg_ncomp(l);
    int64_t n = g.n_el, m = nc * n;
    if (m > 4096) return uwg_set_error(c, UWG_ERR_ARG, "coarsest pressure level too large for a dense solve");
    double *A = nullptr, *B = nullptr;
    UWG_CUDA(c, cudaMallocAsync((void**)&A, sizeof(double) * m * m, c->stream));
    UWG_CUDA(c, cudaMallocAsync((void**)&B, sizeof(double) * m * m, c->stream));
    UWG_CUDA(c, cudaMemsetAsync(A, 0, sizeof(double) * m * m, c->stream));
    PMG_DIM_NC(k_pdense, nc, nblk(n, 64), g, st, A);
    k_pdense_fix<<<1, 1024, 0, c->stream>>>(m, n, fix_checkerboard, g.res[0], g.res[1], A);
    int rc = uwg_ops_dense_invert(c, m, A, B);
    if (!rc) rc = uwg_ops_to_f32(c, m * m, B, inv32);
    cudaFreeAsync(A, c->stream);
    cudaFreeAsync(B, c->stream);
    if (rc) return rc;
    UWG_CUDA(c, cudaGetLastError());
    return UWG_OK;
}
