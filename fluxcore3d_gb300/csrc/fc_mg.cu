// fc_mg.cu -- geometric-multigrid kernels for the thermal advection-diffusion
// operator (sm_103a), behind a C ABI.
//
// Operator (reference solver/nlevel_mg_cuda.py:417-507 and mg_kernels.cu:55-106):
//   L(T)_c = diagL_c T_c - sum_n a_n,c T_n          (7-point, per-cell a_E..a_D)
//   M(T)   = T + dt L(T)                             ("mop")
// with diagL = sum_n a_n.  Every kernel here evaluates L in the equivalent
// flux form sum_n a_n,c (T_c - T_n): in FP32 the rounded diagL differs from the
// sum of the rounded a_n by up to an ulp, so the reference's form applies a
// spurious source (diagL - sum a_n) T_c that is proportional to the absolute
// temperature (T ~ 25 against a rise of ~2) and biases the steady state by a
// few 1e-6 relative; the flux form is exact on constant fields.  diagL is still
// used for the Jacobi weights, as in the reference.
// Ghost cells: the high face of every axis mirrors the cell below it; the low
// face mirrors the cell above it except on the flow axis when the inlet sits at
// index 0, where the cell itself is the ghost (mg_kernels.cu:37-44).
//
// Kernels: the reference pair (mop, jacobi) plus fused forms used by the
// V-cycle: one Jacobi sweep in a single pass (x_out = x + invD (b - M x)),
// the first sweep from a zero guess (x = invD b), residual + 2x mean
// restriction, trilinear prolongation + damped correction + mask, and the
// operator / hierarchy builders.  Reductions are FP64 with a fixed tree order.
#include <initializer_list>

#include "fc_common.cuh"
#include "fc_tma.cuh"
#include "../../include/fluxcore3d_gb300.h"

using namespace fc;

namespace {

constexpr int BLOCK = 256;
inline unsigned grid_for(long long n) { return (unsigned)((n + BLOCK - 1) / BLOCK); }

struct Lvl {
    int nx, ny, nz;
    int ax, out_idx;
};

__device__ __forceinline__ int low_ghost(const Lvl& g, int axis) {
    return (g.ax == axis && g.out_idx != 0) ? 0 : 1;
}

// neighbour indices with the operator's ghosting
struct Nb7 {
    long long c, e, w, n, s, u, d;
};
__device__ __forceinline__ Nb7 nb7(const Lvl& g, int i, int j, int k) {
    const int iE = i < g.nx - 1 ? i + 1 : i - 1;
    const int iW = i > 0 ? i - 1 : low_ghost(g, 0);
    const int jN = j < g.ny - 1 ? j + 1 : j - 1;
    const int jS = j > 0 ? j - 1 : low_ghost(g, 1);
    const int kU = k < g.nz - 1 ? k + 1 : k - 1;
    const int kD = k > 0 ? k - 1 : low_ghost(g, 2);
    const long long nynz = (long long)g.ny * g.nz;
    Nb7 n;
    n.c = i * nynz + (long long)j * g.nz + k;
    n.e = iE * nynz + (long long)j * g.nz + k;
    n.w = iW * nynz + (long long)j * g.nz + k;
    n.n = i * nynz + (long long)jN * g.nz + k;
    n.s = i * nynz + (long long)jS * g.nz + k;
    n.u = i * nynz + (long long)j * g.nz + kU;
    n.d = i * nynz + (long long)j * g.nz + kD;
    return n;
}

struct Coef {
    const float *aE, *aW, *aN, *aS, *aU, *aD, *diagL;
};

// The 7-point operator and the damped-Jacobi update with every rounding
// explicit (no compiler contraction), so the one-cell, two-cell and
// single-CTA smoothers give the same bits:
//   L  = aE*(xc-xe) + aW*(xc-xw) + aN*(xc-xn) + aS*(xc-xs) + aU*(xc-xu) + aD*(xc-xd)
//        (left to right, each product fused into the running sum)
//   lo = xc + dt*L,  x' = xc + inv*(b - lo),  r = b - lo.
__device__ __forceinline__ float stencil_L(float xc, float ae, float xe, float aw, float xw, float an, float xn,
                                           float as, float xs, float au, float xu, float ad, float xd) {
    float s = __fmul_rn(ae, __fsub_rn(xc, xe));
    s = __fmaf_rn(aw, __fsub_rn(xc, xw), s);
    s = __fmaf_rn(an, __fsub_rn(xc, xn), s);
    s = __fmaf_rn(as, __fsub_rn(xc, xs), s);
    s = __fmaf_rn(au, __fsub_rn(xc, xu), s);
    return __fmaf_rn(ad, __fsub_rn(xc, xd), s);
}
__device__ __forceinline__ float m_apply(float xc, float dt, float L) { return __fmaf_rn(dt, L, xc); }
__device__ __forceinline__ float jacobi(float xc, float iv, float bc, float lo) {
    return __fmaf_rn(iv, __fsub_rn(bc, lo), xc);
}

__device__ __forceinline__ float apply_Lf(const Coef& a, const float* __restrict__ x, const Nb7& n, float xc) {
    return stencil_L(xc, __ldg(a.aE + n.c), x[n.e], __ldg(a.aW + n.c), x[n.w],
                     __ldg(a.aN + n.c), x[n.n], __ldg(a.aS + n.c), x[n.s], __ldg(a.aU + n.c), x[n.u],
                     __ldg(a.aD + n.c), x[n.d]);
}


// (levels hold fewer than 2^31 cells: 32-bit index arithmetic)
__device__ __forceinline__ void coords(const Lvl& g, long long idx, int& i, int& j, int& k) {
    const int id = (int)idx;
    const int nynz = g.ny * g.nz;
    i = id / nynz;
    const int r = id - i * nynz;
    j = r / g.nz;
    k = r - j * g.nz;
}

// ---- reference pair -------------------------------------------------------
__global__ void __launch_bounds__(BLOCK) k_mop(const float* __restrict__ T, Coef a, float* __restrict__ Lo,
                                               float dt, Lvl g) {
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (long long)g.nx * g.ny * g.nz) return;
    int i, j, k;
    coords(g, idx, i, j, k);
    const Nb7 n = nb7(g, i, j, k);
    const float tc = T[idx];
    Lo[idx] = m_apply(tc, dt, apply_Lf(a, T, n, tc));
}

__global__ void __launch_bounds__(BLOCK) k_jacobi(float* __restrict__ x, const float* __restrict__ b,
                                                  const float* __restrict__ Lo, const float* __restrict__ inv,
                                                  long long n) {
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= n) return;
    x[idx] += inv[idx] * (b[idx] - Lo[idx]);
}

// L(T) = (M(T) - T) / dt, evaluated the way the reference's L_apply_fine does
__global__ void __launch_bounds__(BLOCK) k_apply_L(const float* __restrict__ T, Coef a, float* __restrict__ out,
                                                   float dt, Lvl g) {
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (long long)g.nx * g.ny * g.nz) return;
    int i, j, k;
    coords(g, idx, i, j, k);
    const Nb7 n = nb7(g, i, j, k);
    const float tc = T[idx];
    const float lo = m_apply(tc, dt, apply_Lf(a, T, n, tc));
    out[idx] = (lo - tc) / dt;
}

// ---- fused V-cycle pieces ------------------------------------------------
__global__ void __launch_bounds__(BLOCK) k_smooth(const float* __restrict__ x, float* __restrict__ xo,
                                                  const float* __restrict__ b, const float* __restrict__ inv,
                                                  Coef a, float dt, Lvl g) {
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (long long)g.nx * g.ny * g.nz) return;
    int i, j, k;
    coords(g, idx, i, j, k);
    const Nb7 n = nb7(g, i, j, k);
    const float tc = x[idx];
    xo[idx] = jacobi(tc, __ldg(inv + idx), __ldg(b + idx), m_apply(tc, dt, apply_Lf(a, x, n, tc)));
}

__global__ void __launch_bounds__(BLOCK) k_smooth_zero(float* __restrict__ xo, const float* __restrict__ b,
                                                       const float* __restrict__ inv, long long n) {
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= n) return;
    xo[idx] = jacobi(0.f, inv[idx], b[idx], 0.f);
}

// The first two sweeps from a zero guess in one pass: x1 = invD b is formed on
// the fly for the cell and its six neighbours, then x2 = x1 + invD (b - M x1).
__global__ void __launch_bounds__(BLOCK) k_smooth_first2(float* __restrict__ xo, const float* __restrict__ b,
                                                         const float* __restrict__ inv, Coef a, float dt, Lvl g) {
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (long long)g.nx * g.ny * g.nz) return;
    int i, j, k;
    coords(g, idx, i, j, k);
    const Nb7 nb = nb7(g, i, j, k);
    auto x1 = [&](long long q) { return jacobi(0.f, __ldg(inv + q), __ldg(b + q), 0.f); };
    const float tc = x1(nb.c);
    const float L = stencil_L(tc, __ldg(a.aE + nb.c), x1(nb.e), __ldg(a.aW + nb.c), x1(nb.w),
                              __ldg(a.aN + nb.c), x1(nb.n), __ldg(a.aS + nb.c), x1(nb.s), __ldg(a.aU + nb.c),
                              x1(nb.u), __ldg(a.aD + nb.c), x1(nb.d));
    xo[idx] = jacobi(tc, __ldg(inv + idx), __ldg(b + idx), m_apply(tc, dt, L));
}

// ---- two cells per thread along k ------------------------------------------
// Levels with an even nz: a thread owns cells (k, k+1) of one row, loads every
// field as float2 and reuses the pair for each other's z neighbour.  Block =
// 32 pairs x 4 rows; grid (nz/64, ny/4, nx) -- no index division.  Same
// arithmetic per cell as k_smooth / k_smooth_first2.
constexpr int PAIR_X = 32, PAIR_Y = 4;

struct PairNb {
    int c, e, w, n, s, d0, u1;   // row-major offsets: centre pair, lateral pairs, z neighbours outside the pair
};
__device__ __forceinline__ PairNb pair_nb(const Lvl& g, int i, int j, int k) {
    const int iE = i < g.nx - 1 ? i + 1 : i - 1, iW = i > 0 ? i - 1 : low_ghost(g, 0);
    const int jN = j < g.ny - 1 ? j + 1 : j - 1, jS = j > 0 ? j - 1 : low_ghost(g, 1);
    const int kD = k > 0 ? k - 1 : low_ghost(g, 2);
    const int kU = k + 2 < g.nz ? k + 2 : k;     // cell k+1's upper neighbour (mirror at the top)
    const int nyz = g.ny * g.nz;
    PairNb p;
    p.c = i * nyz + j * g.nz + k;
    p.e = iE * nyz + j * g.nz + k;
    p.w = iW * nyz + j * g.nz + k;
    p.n = i * nyz + jN * g.nz + k;
    p.s = i * nyz + jS * g.nz + k;
    p.d0 = i * nyz + j * g.nz + kD;
    p.u1 = i * nyz + j * g.nz + kU;
    return p;
}
__device__ __forceinline__ float2 ld2(const float* __restrict__ p, int o) {
    return __ldg(reinterpret_cast<const float2*>(p + o));
}

template <bool FROM_ZERO>
__global__ void __launch_bounds__(PAIR_X * PAIR_Y) k_smooth2(const float* __restrict__ x, float* __restrict__ xo,
                                                             const float* __restrict__ b,
                                                             const float* __restrict__ inv, Coef a, float dt, Lvl g) {
    const int k = 2 * (blockIdx.x * PAIR_X + threadIdx.x);
    const int j = blockIdx.y * PAIR_Y + threadIdx.y;
    const int i = blockIdx.z;
    if (k >= g.nz || j >= g.ny) return;
    const PairNb p = pair_nb(g, i, j, k);
    // the iterate at a pair position (or, from zero, the first sweep's value there)
    auto X2 = [&](int o) -> float2 {
        if (FROM_ZERO) {
            const float2 iv = ld2(inv, o), bb = ld2(b, o);
            return make_float2(jacobi(0.f, iv.x, bb.x, 0.f), jacobi(0.f, iv.y, bb.y, 0.f));
        }
        return *reinterpret_cast<const float2*>(x + o);
    };
    auto X1 = [&](int o) -> float {
        if (FROM_ZERO) return jacobi(0.f, __ldg(inv + o), __ldg(b + o), 0.f);
        return x[o];
    };
    const float2 xc = X2(p.c), xe = X2(p.e), xw = X2(p.w), xn = X2(p.n), xs = X2(p.s);
    const float xd0 = X1(p.d0), xu1 = X1(p.u1);
    const float2 ae = ld2(a.aE, p.c), aw = ld2(a.aW, p.c), an = ld2(a.aN, p.c);
    const float2 as = ld2(a.aS, p.c), au = ld2(a.aU, p.c), ad = ld2(a.aD, p.c);
    const float2 iv = ld2(inv, p.c), bc = ld2(b, p.c);
    const float L0 = stencil_L(xc.x, ae.x, xe.x, aw.x, xw.x, an.x, xn.x, as.x, xs.x, au.x, xc.y, ad.x, xd0);
    const float L1 = stencil_L(xc.y, ae.y, xe.y, aw.y, xw.y, an.y, xn.y, as.y, xs.y, au.y, xu1, ad.y, xc.x);
    *reinterpret_cast<float2*>(xo + p.c) = make_float2(jacobi(xc.x, iv.x, bc.x, m_apply(xc.x, dt, L0)),
                                                       jacobi(xc.y, iv.y, bc.y, m_apply(xc.y, dt, L1)));
}

// All sweeps of a level small enough for one CTA (the coarsest level): the
// iterate ping-pongs in shared memory, each sweep the same arithmetic as
// k_smooth (the first one as k_smooth_zero when starting from zero).
constexpr int SMALL_THREADS = 1024;
constexpr int SMALL_MAX_CELLS = 6144;   // 2 x 24 KB of shared memory, below the 48 KB default

__global__ void __launch_bounds__(SMALL_THREADS) k_smooth_small(float* __restrict__ x, const float* __restrict__ b,
                                                               const float* __restrict__ inv, Coef a, float dt,
                                                               Lvl g, int n_sweeps, int from_zero) {
    extern __shared__ float xs[];
    const int n = g.nx * g.ny * g.nz;
    float* cur = xs;
    float* nxt = xs + n;
    int s0 = 0;
    for (int c = threadIdx.x; c < n; c += blockDim.x) {
        if (from_zero) cur[c] = jacobi(0.f, inv[c], b[c], 0.f);
        else cur[c] = x[c];
    }
    if (from_zero) s0 = 1;
    __syncthreads();
    if (n <= SMALL_THREADS) {
        // one cell per thread: its coefficients and neighbour offsets stay in registers
        const int c = threadIdx.x;
        const bool act = c < n;
        Nb7 nb{0, 0, 0, 0, 0, 0, 0};
        float ae = 0.f, aw = 0.f, an = 0.f, as = 0.f, au = 0.f, ad = 0.f, iv = 0.f, bc = 0.f;
        if (act) {
            int i, j, k;
            coords(g, c, i, j, k);
            nb = nb7(g, i, j, k);
            ae = __ldg(a.aE + c); aw = __ldg(a.aW + c); an = __ldg(a.aN + c);
            as = __ldg(a.aS + c); au = __ldg(a.aU + c); ad = __ldg(a.aD + c);
            iv = __ldg(inv + c); bc = __ldg(b + c);
        }
        for (int sw = s0; sw < n_sweeps; ++sw) {
            if (act) {
                const float tc = cur[c];
                const float L = stencil_L(tc, ae, cur[nb.e], aw, cur[nb.w], an, cur[nb.n], as, cur[nb.s], au,
                                          cur[nb.u], ad, cur[nb.d]);
                nxt[c] = jacobi(tc, iv, bc, m_apply(tc, dt, L));
            }
            __syncthreads();
            float* t = cur;
            cur = nxt;
            nxt = t;
        }
    } else {
        for (int sw = s0; sw < n_sweeps; ++sw) {
            for (int c = threadIdx.x; c < n; c += blockDim.x) {
                int i, j, k;
                coords(g, c, i, j, k);
                const Nb7 nb = nb7(g, i, j, k);
                const float tc = cur[c];
                nxt[c] = jacobi(tc, __ldg(inv + c), __ldg(b + c), m_apply(tc, dt, apply_Lf(a, cur, nb, tc)));
            }
            __syncthreads();
            float* t = cur;
            cur = nxt;
            nxt = t;
        }
    }
    for (int c = threadIdx.x; c < n; c += blockDim.x) x[c] = cur[c];
}

// coarse b = mean over each 2x2x2 block of r = mask * (b - M x); fine cells
// beyond the even-cropped extent do not contribute (view(...).mean semantics)
__global__ void __launch_bounds__(BLOCK) k_residual_restrict(const float* __restrict__ x, const float* __restrict__ b,
                                                             const float* __restrict__ mask, Coef a, float dt, Lvl g,
                                                             float* __restrict__ bc, int cx, int cy, int cz) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (long long)cx * cy * cz) return;
    const int cyz = cy * cz;
    const int ic = (int)t / cyz;
    const int rr = (int)t - ic * cyz;
    const int jc = rr / cz, kc = rr - jc * cz;
    float s = 0.f;
#pragma unroll
    for (int di = 0; di < 2; ++di)
#pragma unroll
        for (int dj = 0; dj < 2; ++dj)
#pragma unroll
            for (int dk = 0; dk < 2; ++dk) {
                const int i = 2 * ic + di, j = 2 * jc + dj, k = 2 * kc + dk;
                const Nb7 n = nb7(g, i, j, k);
                const float tc = x[n.c];
                const float lo = m_apply(tc, dt, apply_Lf(a, x, n, tc));
                s += __fmul_rn(__fsub_rn(__ldg(b + n.c), lo), __ldg(mask + n.c));
            }
    bc[t] = s * 0.125f;
}

// The same restriction with one thread per fine cell: a block covers 64 fine k
// x 2 fine j x 2 fine i of one coarse (jc, ic) column; k pairs are summed by a
// shuffle, the four (j, i) partials in shared memory.  Full parallelism on the
// coarse levels, where one thread per coarse cell leaves too few threads to
// hide the latency of its eight stencils.  Sum order per coarse cell:
// ((s00 + s01) + s10) + s11 with s_ji = r(k) + r(k+1).
__global__ void __launch_bounds__(256) k_residual_restrict2(const float* __restrict__ x, const float* __restrict__ b,
                                                            const float* __restrict__ mask, Coef a, float dt, Lvl g,
                                                            float* __restrict__ bc, int cx, int cy, int cz) {
    __shared__ float part[4][32];
    const int t = threadIdx.x;
    const int kk = t & 63, dj = (t >> 6) & 1, di = t >> 7;
    const int k = blockIdx.x * 64 + kk;
    const int jc = blockIdx.y, ic = blockIdx.z;
    const int j = 2 * jc + dj, i = 2 * ic + di;
    float r = 0.f;
    if (k < 2 * cz) {
        const Nb7 n = nb7(g, i, j, k);
        const float tc = x[n.c];
        const float lo = m_apply(tc, dt, apply_Lf(a, x, n, tc));
        r = __fmul_rn(__fsub_rn(__ldg(b + n.c), lo), __ldg(mask + n.c));
    }
    r = __fadd_rn(r, __shfl_xor_sync(0xffffffffu, r, 1));
    if ((kk & 1) == 0) part[(di << 1) | dj][kk >> 1] = r;
    __syncthreads();
    if (t < 32) {
        const int kc = blockIdx.x * 32 + t;
        if (kc < cz) {
            const float s = __fadd_rn(__fadd_rn(__fadd_rn(part[0][t], part[1][t]), part[2][t]), part[3][t]);
            bc[((long long)ic * cy + jc) * cz + kc] = __fmul_rn(s, 0.125f);
        }
    }
}

// trilinear (align_corners = False) source coordinate of fine index i
__device__ __forceinline__ void src_coord(int i, int nf, int nc, int& i0, int& i1, float& l1) {
    const float scale = (float)nc / (float)nf;
    float s = scale * ((float)i + 0.5f) - 0.5f;
    if (s < 0.f) s = 0.f;
    i0 = (int)s;
    if (i0 > nc - 1) i0 = nc - 1;
    i1 = i0 + (i0 < nc - 1 ? 1 : 0);
    l1 = s - (float)i0;
}

__global__ void __launch_bounds__(BLOCK) k_prolong_correct(float* __restrict__ x, const float* __restrict__ xc,
                                                           const float* __restrict__ mask, int nx, int ny, int nz,
                                                           int cx, int cy, int cz, float alpha) {
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (long long)nx * ny * nz) return;
    const int nyz = ny * nz;
    const int i = (int)idx / nyz;
    const int r = (int)idx - i * nyz;
    const int j = r / nz, k = r - j * nz;
    int i0, i1, j0, j1, k0, k1;
    float li, lj, lk;
    src_coord(i, nx, cx, i0, i1, li);
    src_coord(j, ny, cy, j0, j1, lj);
    src_coord(k, nz, cz, k0, k1, lk);
    const float hi = 1.f - li, hj = 1.f - lj, hk = 1.f - lk;
    auto X = [&](int a, int b, int c) { return __ldg(xc + ((long long)a * cy + b) * cz + c); };
    const float e = hi * (hj * (hk * X(i0, j0, k0) + lk * X(i0, j0, k1)) + lj * (hk * X(i0, j1, k0) + lk * X(i0, j1, k1))) +
                    li * (hj * (hk * X(i1, j0, k0) + lk * X(i1, j0, k1)) + lj * (hk * X(i1, j1, k0) + lk * X(i1, j1, k1)));
    x[idx] = (x[idx] + alpha * e) * __ldg(mask + idx);
}

// Exact 2:1 coarsening on every axis (nf = 2 nc): the align_corners = False
// source coordinate is 0.5 i - 0.25 exactly, so i = 2m gives (m - 1, m, 0.75)
// (m = 0: (0, 0, 0) after the clamp at 0) and i = 2m + 1 gives (m, m + 1, 0.25)
// (m + 1 clamped to nc - 1) -- the same values src_coord computes.  3D launch:
// x = k, y = j, z = i, so no index division.
__device__ __forceinline__ void src_2to1(int i, int nc, int& i0, int& i1, float& l1) {
    const int m = i >> 1;
    if (i & 1) {
        i0 = m;
        i1 = m + 1 < nc ? m + 1 : m;
        l1 = 0.25f;
    } else if (m == 0) {
        i0 = 0;
        i1 = nc > 1 ? 1 : 0;
        l1 = 0.f;
    } else {
        i0 = m - 1;
        i1 = m;
        l1 = 0.75f;
    }
}

// trilinear interpolation of the coarse correction at one fine cell of an exact
// 2:1 coarsening, then x = (x + alpha e) mask, every rounding explicit
__device__ __forceinline__ float prolong_cell(const float* __restrict__ xc, int cy, int cz, int i, int j, int k, int cx,
                                              float xv, float m, float alpha) {
    int i0, i1, j0, j1, k0, k1;
    float li, lj, lk;
    src_2to1(i, cx, i0, i1, li);
    src_2to1(j, cy, j0, j1, lj);
    src_2to1(k, cz, k0, k1, lk);
    const float hi = 1.f - li, hj = 1.f - lj, hk = 1.f - lk;
    const int p0 = i0 * cy * cz, p1 = i1 * cy * cz, r0 = j0 * cz, r1 = j1 * cz;
    auto X = [&](int p, int r, int c) { return __ldg(xc + p + r + c); };
    auto zl = [&](int p, int r) { return __fmaf_rn(lk, X(p, r, k1), __fmul_rn(hk, X(p, r, k0))); };
    const float y0 = __fmaf_rn(lj, zl(p0, r1), __fmul_rn(hj, zl(p0, r0)));
    const float y1 = __fmaf_rn(lj, zl(p1, r1), __fmul_rn(hj, zl(p1, r0)));
    const float e = __fmaf_rn(li, y1, __fmul_rn(hi, y0));
    return __fmul_rn(__fmaf_rn(alpha, e, xv), m);
}

__global__ void __launch_bounds__(BLOCK) k_prolong_2to1(float* __restrict__ x, const float* __restrict__ xc,
                                                        const float* __restrict__ mask, int nx, int ny, int nz,
                                                        int cx, int cy, int cz, float alpha) {
    const int k = blockIdx.x * 64 + (threadIdx.x & 63);
    const int j = blockIdx.y * 4 + (threadIdx.x >> 6);
    const int i = blockIdx.z;
    if (k >= nz || j >= ny) return;
    const int idx = (i * ny + j) * nz + k;
    x[idx] = prolong_cell(xc, cy, cz, i, j, k, cx, x[idx], __ldg(mask + idx), alpha);
}

// k_prolong_2to1 on two cells (k, k+1) per thread (nz even): float2 update of
// x and float2 mask; the same interpolation per cell.
__global__ void __launch_bounds__(PAIR_X * PAIR_Y) k_prolong2(float* __restrict__ x, const float* __restrict__ xc,
                                                              const float* __restrict__ mask, int nx, int ny, int nz,
                                                              int cx, int cy, int cz, float alpha) {
    const int k = 2 * (blockIdx.x * PAIR_X + threadIdx.x);
    const int j = blockIdx.y * PAIR_Y + threadIdx.y;
    const int i = blockIdx.z;
    if (k >= nz || j >= ny) return;
    const int idx = (i * ny + j) * nz + k;
    float2* xp = reinterpret_cast<float2*>(x + idx);
    const float2 xv = *xp, m = __ldg(reinterpret_cast<const float2*>(mask + idx));
    *xp = make_float2(prolong_cell(xc, cy, cz, i, j, k, cx, xv.x, m.x, alpha),
                      prolong_cell(xc, cy, cz, i, j, k + 1, cx, xv.y, m.y, alpha));
}

// k_prolong_2to1 on four cells (k .. k+3) per thread (nz a multiple of 4):
// float4 update of x and float4 mask, the same interpolation per cell; the four
// cells read coarse columns m-1 .. m+2 of their two planes and two rows, which
// the compiler loads once for all four.
__global__ void __launch_bounds__(PAIR_X * PAIR_Y) k_prolong4(float* __restrict__ x, const float* __restrict__ xc,
                                                              const float* __restrict__ mask, int nx, int ny, int nz,
                                                              int cx, int cy, int cz, float alpha) {
    const int k = 4 * (blockIdx.x * PAIR_X + threadIdx.x);
    const int j = blockIdx.y * PAIR_Y + threadIdx.y;
    const int i = blockIdx.z;
    if (k >= nz || j >= ny) return;
    const int idx = (i * ny + j) * nz + k;
    float4* xp = reinterpret_cast<float4*>(x + idx);
    const float4 xv = *xp, m = __ldg(reinterpret_cast<const float4*>(mask + idx));
    *xp = make_float4(prolong_cell(xc, cy, cz, i, j, k, cx, xv.x, m.x, alpha),
                      prolong_cell(xc, cy, cz, i, j, k + 1, cx, xv.y, m.y, alpha),
                      prolong_cell(xc, cy, cz, i, j, k + 2, cx, xv.z, m.z, alpha),
                      prolong_cell(xc, cy, cz, i, j, k + 3, cx, xv.w, m.w, alpha));
}

// TMA-staged prolongation of an exact 2:1 coarsening (nz a multiple of 8, at
// most 256): a CTA corrects R whole fine rows of one fine plane i (R = 2 *
// max(1, 256 / nz), so R nz <= 512 cells, four per thread).  Everything those
// cells interpolate from -- coarse planes pl, pl+1 and coarse rows
// j0/2 - 1 .. (j0 + R)/2, every column -- arrives in shared memory with one
// tensor copy (rows or planes outside the level read as zero and are never
// used: src_2to1 clamps to the level), so the eight-point stencils read shared
// memory instead of L1.  The fine x and mask move as float4.  The same
// roundings as prolong_cell, so the result equals k_prolong4's bit for bit.
// If the copy's bounded wait gives up, the CTA interpolates from global memory
// instead (same result) and waits again, bounded, before it retires.
constexpr int PT_THREADS = 128;

__device__ __forceinline__ float prolong_cell_tile(const float* __restrict__ tile, int pl, int jc0, int rows, int cy,
                                                   int cz, int i, int j, int k, int cx, float xv, float m,
                                                   float alpha) {
    int i0, i1, j0, j1, k0, k1;
    float li, lj, lk;
    src_2to1(i, cx, i0, i1, li);
    src_2to1(j, cy, j0, j1, lj);
    src_2to1(k, cz, k0, k1, lk);
    const float hi = 1.f - li, hj = 1.f - lj, hk = 1.f - lk;
    const int p0 = (i0 - pl) * rows * cz, p1 = (i1 - pl) * rows * cz, r0 = (j0 - jc0) * cz, r1 = (j1 - jc0) * cz;
    auto X = [&](int p, int r, int c) { return tile[p + r + c]; };
    auto zl = [&](int p, int r) { return __fmaf_rn(lk, X(p, r, k1), __fmul_rn(hk, X(p, r, k0))); };
    const float y0 = __fmaf_rn(lj, zl(p0, r1), __fmul_rn(hj, zl(p0, r0)));
    const float y1 = __fmaf_rn(lj, zl(p1, r1), __fmul_rn(hj, zl(p1, r0)));
    const float e = __fmaf_rn(li, y1, __fmul_rn(hi, y0));
    return __fmul_rn(__fmaf_rn(alpha, e, xv), m);
}

__global__ void __launch_bounds__(PT_THREADS) k_prolong_tma(const __grid_constant__ CUtensorMap tmc,
                                                            float* __restrict__ x, const float* __restrict__ xc,
                                                            const float* __restrict__ mask, int nx, int ny, int nz,
                                                            int cx, int cy, int cz, int R, float alpha) {
    // [2][rows][cz] coarse floats, then the mbarrier (no static shared memory, so the
    // tile starts on the 128-byte boundary the tensor copy needs)
    extern __shared__ __align__(128) unsigned char pt_smem[];
    float* tile = reinterpret_cast<float*>(pt_smem);
    const int i = blockIdx.y;
    const int jf0 = blockIdx.x * R;
    const int m = i >> 1;
    const int pl = ((i & 1) == 0 && m > 0) ? m - 1 : m;   // first coarse plane of the box
    const int jc0 = (jf0 >> 1) - 1;                       // first coarse row of the box
    const int rows = R / 2 + 2;
    const uint32_t tile_bytes = (uint32_t)(2 * rows * cz) * 4u;   // a multiple of 32 (cz % 4 == 0)
    const uint32_t b = su32(pt_smem + tile_bytes);
    if (threadIdx.x == 0) {
        bar_init(b, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        bar_expect_tx(b, tile_bytes);
        tma_load_3d(su32(tile), &tmc, 0, jc0, pl, b);
    }
    __syncthreads();
    const bool staged = bar_wait(b, 0u);
    const int per_row = nz >> 2;
    const int r = threadIdx.x / per_row;
    const int k = (threadIdx.x - r * per_row) * 4;
    const int j = jf0 + r;
    if (r < R && j < ny) {
        const int idx = (i * ny + j) * nz + k;
        float4* xp = reinterpret_cast<float4*>(x + idx);
        const float4 xv = *xp, mv = __ldg(reinterpret_cast<const float4*>(mask + idx));
        if (staged)
            *xp = make_float4(prolong_cell_tile(tile, pl, jc0, rows, cy, cz, i, j, k, cx, xv.x, mv.x, alpha),
                              prolong_cell_tile(tile, pl, jc0, rows, cy, cz, i, j, k + 1, cx, xv.y, mv.y, alpha),
                              prolong_cell_tile(tile, pl, jc0, rows, cy, cz, i, j, k + 2, cx, xv.z, mv.z, alpha),
                              prolong_cell_tile(tile, pl, jc0, rows, cy, cz, i, j, k + 3, cx, xv.w, mv.w, alpha));
        else
            *xp = make_float4(prolong_cell(xc, cy, cz, i, j, k, cx, xv.x, mv.x, alpha),
                              prolong_cell(xc, cy, cz, i, j, k + 1, cx, xv.y, mv.y, alpha),
                              prolong_cell(xc, cy, cz, i, j, k + 2, cx, xv.z, mv.z, alpha),
                              prolong_cell(xc, cy, cz, i, j, k + 3, cx, xv.w, mv.w, alpha));
    }
    if (!__syncthreads_and(staged) && threadIdx.x == 0) bar_wait(b, 0u);   // let a late copy land first
}

// per-block partial sums of (w * (b - M x))^2 in FP64, w = mask or 1
__global__ void __launch_bounds__(BLOCK) k_residual_sq(const float* __restrict__ x, const float* __restrict__ b,
                                                       const float* __restrict__ mask, Coef a, float dt, Lvl g,
                                                       float* __restrict__ r_out, double* __restrict__ part) {
    __shared__ double sh[BLOCK];
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    double v = 0.0;
    if (idx < (long long)g.nx * g.ny * g.nz) {
        int i, j, k;
        coords(g, idx, i, j, k);
        const Nb7 n = nb7(g, i, j, k);
        const float tc = x[idx];
        const float lo = m_apply(tc, dt, apply_Lf(a, x, n, tc));
        float r = __fsub_rn(__ldg(b + idx), lo);
        if (mask) r = __fmul_rn(r, __ldg(mask + idx));
        if (r_out) r_out[idx] = r;
        v = (double)r * (double)r;
    }
    sh[threadIdx.x] = v;
    __syncthreads();
    for (int s = BLOCK / 2; s > 0; s >>= 1) {
        if ((int)threadIdx.x < s) sh[threadIdx.x] += sh[threadIdx.x + s];
        __syncthreads();
    }
    if (threadIdx.x == 0) part[blockIdx.x] = sh[0];
}

// Heat-balance integrals in FP64 over the non-Dirichlet cells (mask != 0):
// part[3 b + 0] = sum src, [3 b + 1] = sum L(T) (the operator's net outflow of
// heat, boundary fluxes included), [3 b + 2] = sum T.  L in FP64 (flux form)
// from the FP32 coefficients and temperatures.
__global__ void __launch_bounds__(BLOCK) k_heat_balance(const float* __restrict__ T, const float* __restrict__ src,
                                                        const float* __restrict__ mask, Coef a, Lvl g,
                                                        double* __restrict__ part) {
    __shared__ double sh[3][BLOCK];
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    double vs = 0.0, vl = 0.0, vt = 0.0;
    if (idx < (long long)g.nx * g.ny * g.nz && __ldg(mask + idx) != 0.f) {
        int i, j, k;
        coords(g, idx, i, j, k);
        const Nb7 n = nb7(g, i, j, k);
        const double tc = T[idx];
        vl = (double)__ldg(a.aE + idx) * (tc - (double)T[n.e]) + (double)__ldg(a.aW + idx) * (tc - (double)T[n.w]) +
             (double)__ldg(a.aN + idx) * (tc - (double)T[n.n]) + (double)__ldg(a.aS + idx) * (tc - (double)T[n.s]) +
             (double)__ldg(a.aU + idx) * (tc - (double)T[n.u]) + (double)__ldg(a.aD + idx) * (tc - (double)T[n.d]);
        vs = src ? (double)__ldg(src + idx) : 0.0;
        vt = tc;
    }
    sh[0][threadIdx.x] = vs;
    sh[1][threadIdx.x] = vl;
    sh[2][threadIdx.x] = vt;
    __syncthreads();
    for (int st = BLOCK / 2; st > 0; st >>= 1) {
        if ((int)threadIdx.x < st)
            for (int c = 0; c < 3; ++c) sh[c][threadIdx.x] += sh[c][threadIdx.x + st];
        __syncthreads();
    }
    if (threadIdx.x < 3) part[3 * (long long)blockIdx.x + threadIdx.x] = sh[threadIdx.x][0];
}

// column c of an [n][3] partial array summed in fixed order by one block
__global__ void __launch_bounds__(BLOCK) k_sum_partials3(const double* __restrict__ part, int n,
                                                         double* __restrict__ out) {
    __shared__ double sh[BLOCK];
    for (int c = 0; c < 3; ++c) {
        double v = 0.0;
        for (int p = threadIdx.x; p < n; p += BLOCK) v += part[3 * p + c];
        sh[threadIdx.x] = v;
        __syncthreads();
        for (int s = BLOCK / 2; s > 0; s >>= 1) {
            if ((int)threadIdx.x < s) sh[threadIdx.x] += sh[threadIdx.x + s];
            __syncthreads();
        }
        if (threadIdx.x == 0) out[c] = sh[0];
        __syncthreads();
    }
}

// sum of partials in fixed order by one block
__global__ void __launch_bounds__(BLOCK) k_sum_partials(const double* __restrict__ part, int n, double* __restrict__ out) {
    __shared__ double sh[BLOCK];
    double v = 0.0;
    for (int p = threadIdx.x; p < n; p += BLOCK) v += part[p];
    sh[threadIdx.x] = v;
    __syncthreads();
    for (int s = BLOCK / 2; s > 0; s >>= 1) {
        if ((int)threadIdx.x < s) sh[threadIdx.x] += sh[threadIdx.x + s];
        __syncthreads();
    }
    if (threadIdx.x == 0) *out = sh[0];
}

// ---- operator / hierarchy builders ---------------------------------------
// Harmonic-mean face conductivity, diffusion s k_f /(rho cp dx^2), first-order
// upwind convection s max(+-u, 0)/dx (nlevel_mg_cuda.py:417-507), evaluated as
// separately rounded FP32 operations in the reference's order.
__global__ void __launch_bounds__(BLOCK) k_build_coeffs(const float* __restrict__ kk, const float* __restrict__ rcp,
                                                        const float* __restrict__ u, const float* __restrict__ v,
                                                        const float* __restrict__ w, Lvl g, float cd, float ca,
                                                        float* aE, float* aW, float* aN, float* aS, float* aU,
                                                        float* aD, float* diagL) {
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (long long)g.nx * g.ny * g.nz) return;
    int i, j, k;
    coords(g, idx, i, j, k);
    const Nb7 n = nb7(g, i, j, k);
    const float kc = kk[idx];
    const float inv_rcp = __fdiv_rn(1.0f, __fadd_rn(rcp[idx], 1e-30f));
    auto hm = [&](long long o) {
        const float kn = kk[o];
        return __fdiv_rn(__fmul_rn(__fmul_rn(2.0f, kc), kn), __fadd_rn(__fadd_rn(kc, kn), 1e-30f));
    };
    auto dif = [&](long long o) { return __fmul_rn(__fmul_rn(cd, hm(o)), inv_rcp); };
    const float uc = u[idx], vc = v[idx], wc = w[idx];
    const float upx = fmaxf(uc, 0.f), umx = fmaxf(-uc, 0.f);
    const float upy = fmaxf(vc, 0.f), umy = fmaxf(-vc, 0.f);
    const float upz = fmaxf(wc, 0.f), umz = fmaxf(-wc, 0.f);
    const float e = __fadd_rn(dif(n.e), __fmul_rn(ca, umx));
    const float ww = __fadd_rn(dif(n.w), __fmul_rn(ca, upx));
    const float no = __fadd_rn(dif(n.n), __fmul_rn(ca, umy));
    const float so = __fadd_rn(dif(n.s), __fmul_rn(ca, upy));
    const float up = __fadd_rn(dif(n.u), __fmul_rn(ca, umz));
    const float dn = __fadd_rn(dif(n.d), __fmul_rn(ca, upz));
    aE[idx] = e; aW[idx] = ww; aN[idx] = no; aS[idx] = so; aU[idx] = up; aD[idx] = dn;
    diagL[idx] = __fadd_rn(__fadd_rn(__fadd_rn(__fadd_rn(__fadd_rn(e, ww), no), so), up), dn);
}

// 2x mean restriction of a field (even-cropped); mask variant thresholds at 0.999
__global__ void __launch_bounds__(BLOCK) k_restrict_mean(const float* __restrict__ src, int nx, int ny, int nz,
                                                         float* __restrict__ dst, int cx, int cy, int cz, int as_mask) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (long long)cx * cy * cz) return;
    const int ic = (int)(t / ((long long)cy * cz));
    const int rr = (int)(t - (long long)ic * cy * cz);
    const int jc = rr / cz, kc = rr - (rr / cz) * cz;
    float s = 0.f;
    for (int di = 0; di < 2; ++di)
        for (int dj = 0; dj < 2; ++dj)
            for (int dk = 0; dk < 2; ++dk)
                s += src[((long long)(2 * ic + di) * ny + (2 * jc + dj)) * nz + (2 * kc + dk)];
    const float m = s * 0.125f;
    dst[t] = as_mask ? (m >= 0.999f ? 1.f : 0.f) : m;
}

__global__ void __launch_bounds__(BLOCK) k_inv_diag(const float* __restrict__ diagL, const float* __restrict__ mask,
                                                    float* __restrict__ inv, float dt, float omega, long long n) {
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= n) return;
    float d = 1.0f + dt * diagL[idx];
    d = fmaxf(d, 1e-12f);
    inv[idx] = (omega / d) * mask[idx];
}

// ---- FP64 exact solve of the coarsest level ---------------------------------
// A = I + dt L of the level in FP64 (built from the FP32 couplings with the
// operator's ghosting, diagonal = 1 + dt sum_n a_n as in the flux form; rows of
// Dirichlet cells are identity rows), inverted in place by Gauss-Jordan
// elimination without pivoting: A is strictly diagonally dominant by rows
// (1 + dt sum_n a_n against dt sum_n a_n), so every pivot is positive and no
// growth occurs.  One launch per pivot updates every element; the pivot row and
// column it needs are double-buffered copies written by the previous launch,
// so no element is read after another thread overwrote it.
constexpr int CD_MAX_CELLS = 4096;
constexpr int CD_TX = 32, CD_TY = 8;

__global__ void __launch_bounds__(BLOCK) k_cd_assemble(Coef a, const float* __restrict__ mask, double dt, Lvl g,
                                                       double* __restrict__ A, int n) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= n) return;
    double* row = A + (long long)c * n;
    if (mask[c] == 0.f) {
        row[c] = 1.0;
        return;
    }
    int i, j, k;
    coords(g, c, i, j, k);
    const Nb7 nb = nb7(g, i, j, k);
    // a ghost neighbour can be the cell itself or another neighbour: accumulate
    const double ae = __ldg(a.aE + c), aw = __ldg(a.aW + c), an = __ldg(a.aN + c);
    const double as = __ldg(a.aS + c), au = __ldg(a.aU + c), ad = __ldg(a.aD + c);
    row[c] += 1.0 + dt * (ae + aw + an + as + au + ad);
    row[nb.e] -= dt * ae;
    row[nb.w] -= dt * aw;
    row[nb.n] -= dt * an;
    row[nb.s] -= dt * as;
    row[nb.u] -= dt * au;
    row[nb.d] -= dt * ad;
}

// row and column 0 into the first buffer pair
__global__ void __launch_bounds__(BLOCK) k_cd_seed(const double* __restrict__ A, int n, double* __restrict__ row,
                                                   double* __restrict__ col) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n) return;
    row[t] = A[t];
    col[t] = A[(long long)t * n];
}

// One Gauss-Jordan step on pivot p (row/col: row p and column p before the step);
// also stores row p+1 and column p+1 after the step into the other buffers.
__global__ void __launch_bounds__(CD_TX * CD_TY) k_cd_pivot(double* __restrict__ A, int n, int p,
                                                             const double* __restrict__ row,
                                                             const double* __restrict__ col,
                                                             double* __restrict__ row_next,
                                                             double* __restrict__ col_next) {
    const int j = blockIdx.x * CD_TX + threadIdx.x;
    const int i = blockIdx.y * CD_TY + threadIdx.y;
    if (i >= n || j >= n) return;
    const double inv = 1.0 / row[p];
    double v;
    if (i == p) v = (j == p) ? inv : row[j] * inv;
    else if (j == p) v = -col[i] * inv;
    else v = fma(-col[i], row[j] * inv, A[(long long)i * n + j]);
    A[(long long)i * n + j] = v;
    if (i == p + 1) row_next[j] = v;
    if (j == p + 1) col_next[i] = v;
}

// x_i = mask_i * sum_j inv_ij mask_j b_j in FP64: one warp per row, b staged in shared memory
__global__ void __launch_bounds__(256) k_cd_apply(const double* __restrict__ inv, const float* __restrict__ b,
                                                  const float* __restrict__ mask, float* __restrict__ x, int n) {
    extern __shared__ double bs[];
    for (int t = threadIdx.x; t < n; t += blockDim.x) bs[t] = mask[t] != 0.f ? (double)b[t] : 0.0;
    __syncthreads();
    const int row = blockIdx.x * 8 + (threadIdx.x >> 5);
    const int lane = threadIdx.x & 31;
    if (row >= n) return;
    const double* r = inv + (long long)row * n;
    double s = 0.0;
    for (int j = lane; j < n; j += 32) s = fma(__ldg(r + j), bs[j], s);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if (lane == 0) x[row] = mask[row] != 0.f ? (float)s : 0.f;
}

int level_ok(const Lvl& g) {
    if (g.nx < 2 || g.ny < 2 || g.nz < 2) return FC_ERR_ARG;
    if ((long long)g.nx * g.ny * g.nz >= (1LL << 31)) return FC_ERR_ARG;
    if (g.ax < 0 || g.ax > 2) return FC_ERR_ARG;
    return FC_OK;
}

}  // namespace

// two-cells-per-thread path: even nz, 8-byte aligned fields, grid within limits
static bool pair_ok(const Lvl& g, std::initializer_list<const float*> ptrs) {
    if (g.nz < 2 || (g.nz & 1) || g.nx > 65535 || (g.ny + PAIR_Y - 1) / PAIR_Y > 65535) return false;
    for (const float* p : ptrs)
        if (reinterpret_cast<uintptr_t>(p) & 7) return false;
    return true;
}
static dim3 pair_grid(const Lvl& g) {
    return dim3((unsigned)((g.nz + 2 * PAIR_X - 1) / (2 * PAIR_X)), (unsigned)((g.ny + PAIR_Y - 1) / PAIR_Y),
                (unsigned)g.nx);
}

extern "C" {

int fc_mg_mop(const float* T, const float* aE, const float* aW, const float* aN, const float* aS, const float* aU,
              const float* aD, const float* diagL, float* Lo, float dt, int nx, int ny, int nz, int ax, int out_idx,
              void* stream) {
    Lvl g{nx, ny, nz, ax, out_idx};
    if (level_ok(g) || !T || !Lo || !aE || !aW || !aN || !aS || !aU || !aD || !diagL) return FC_ERR_ARG;
    Coef a{aE, aW, aN, aS, aU, aD, diagL};
    k_mop<<<grid_for((long long)nx * ny * nz), BLOCK, 0, (cudaStream_t)stream>>>(T, a, Lo, dt, g);
    return launch_status();
}

int fc_mg_jacobi(float* x, const float* b, const float* Lo, const float* inv_diagM, long long n, void* stream) {
    if (!x || !b || !Lo || !inv_diagM || n < 0) return FC_ERR_ARG;
    if (n == 0) return FC_OK;
    k_jacobi<<<grid_for(n), BLOCK, 0, (cudaStream_t)stream>>>(x, b, Lo, inv_diagM, n);
    return launch_status();
}

int fc_mg_apply_L(const float* T, const float* aE, const float* aW, const float* aN, const float* aS,
                  const float* aU, const float* aD, const float* diagL, float* out, float dt, int nx, int ny, int nz,
                  int ax, int out_idx, void* stream) {
    Lvl g{nx, ny, nz, ax, out_idx};
    if (level_ok(g) || !T || !out || dt == 0.f) return FC_ERR_ARG;
    Coef a{aE, aW, aN, aS, aU, aD, diagL};
    k_apply_L<<<grid_for((long long)nx * ny * nz), BLOCK, 0, (cudaStream_t)stream>>>(T, a, out, dt, g);
    return launch_status();
}

int fc_mg_smooth(const float* x_in, float* x_out, const float* b, const float* inv_diagM, const float* aE,
                 const float* aW, const float* aN, const float* aS, const float* aU, const float* aD,
                 const float* diagL, float dt, int nx, int ny, int nz, int ax, int out_idx, void* stream) {
    Lvl g{nx, ny, nz, ax, out_idx};
    if (level_ok(g) || !x_in || !x_out || x_in == x_out || !b || !inv_diagM) return FC_ERR_ARG;
    Coef a{aE, aW, aN, aS, aU, aD, diagL};
    if (pair_ok(g, {x_in, x_out, b, inv_diagM, aE, aW, aN, aS, aU, aD, diagL}))
        k_smooth2<false><<<pair_grid(g), dim3(PAIR_X, PAIR_Y), 0, (cudaStream_t)stream>>>(x_in, x_out, b, inv_diagM,
                                                                                         a, dt, g);
    else
        k_smooth<<<grid_for((long long)nx * ny * nz), BLOCK, 0, (cudaStream_t)stream>>>(x_in, x_out, b, inv_diagM, a,
                                                                                      dt, g);
    return launch_status();
}

int fc_mg_smooth_small(float* x, const float* b, const float* inv_diagM, const float* aE, const float* aW,
                       const float* aN, const float* aS, const float* aU, const float* aD, const float* diagL,
                       float dt, int nx, int ny, int nz, int ax, int out_idx, int n_sweeps, int from_zero,
                       void* stream) {
    Lvl g{nx, ny, nz, ax, out_idx};
    if (level_ok(g) || !x || !b || !inv_diagM || n_sweeps < 1) return FC_ERR_ARG;
    const long long n = (long long)nx * ny * nz;
    if (n > SMALL_MAX_CELLS) return FC_ERR_UNSUPPORTED;
    Coef a{aE, aW, aN, aS, aU, aD, diagL};
    k_smooth_small<<<1, SMALL_THREADS, 2 * n * sizeof(float), (cudaStream_t)stream>>>(x, b, inv_diagM, a, dt, g,
                                                                                     n_sweeps, from_zero != 0);
    return launch_status();
}

int fc_mg_smooth_first2(float* x_out, const float* b, const float* inv_diagM, const float* aE, const float* aW,
                        const float* aN, const float* aS, const float* aU, const float* aD, const float* diagL,
                        float dt, int nx, int ny, int nz, int ax, int out_idx, void* stream) {
    Lvl g{nx, ny, nz, ax, out_idx};
    if (level_ok(g) || !x_out || !b || !inv_diagM || x_out == b) return FC_ERR_ARG;
    Coef a{aE, aW, aN, aS, aU, aD, diagL};
    if (pair_ok(g, {x_out, b, inv_diagM, aE, aW, aN, aS, aU, aD, diagL}))
        k_smooth2<true><<<pair_grid(g), dim3(PAIR_X, PAIR_Y), 0, (cudaStream_t)stream>>>(nullptr, x_out, b, inv_diagM,
                                                                                        a, dt, g);
    else
        k_smooth_first2<<<grid_for((long long)nx * ny * nz), BLOCK, 0, (cudaStream_t)stream>>>(x_out, b, inv_diagM,
                                                                                             a, dt, g);
    return launch_status();
}

int fc_mg_smooth_from_zero(float* x_out, const float* b, const float* inv_diagM, long long n, void* stream) {
    if (!x_out || !b || !inv_diagM || n < 0) return FC_ERR_ARG;
    if (n == 0) return FC_OK;
    k_smooth_zero<<<grid_for(n), BLOCK, 0, (cudaStream_t)stream>>>(x_out, b, inv_diagM, n);
    return launch_status();
}

int fc_mg_residual_restrict(const float* x, const float* b, const float* mask, const float* aE, const float* aW,
                            const float* aN, const float* aS, const float* aU, const float* aD, const float* diagL,
                            float dt, int nx, int ny, int nz, int ax, int out_idx, float* b_coarse, int cx, int cy,
                            int cz, void* stream) {
    Lvl g{nx, ny, nz, ax, out_idx};
    if (level_ok(g) || !x || !b || !mask || !b_coarse) return FC_ERR_ARG;
    if (cx != nx / 2 || cy != ny / 2 || cz != nz / 2 || cx < 1 || cy < 1 || cz < 1) return FC_ERR_ARG;
    Coef a{aE, aW, aN, aS, aU, aD, diagL};
    if (cy <= 65535 && cx <= 65535) {
        const dim3 grid((unsigned)((2 * cz + 63) / 64), (unsigned)cy, (unsigned)cx);
        k_residual_restrict2<<<grid, 256, 0, (cudaStream_t)stream>>>(x, b, mask, a, dt, g, b_coarse, cx, cy, cz);
    } else {
        k_residual_restrict<<<grid_for((long long)cx * cy * cz), BLOCK, 0, (cudaStream_t)stream>>>(
            x, b, mask, a, dt, g, b_coarse, cx, cy, cz);
    }
    return launch_status();
}

}  // extern "C"

namespace {
// Launch the TMA-staged prolongation when the level fits it (returns false, having
// launched nothing, otherwise): nz a multiple of 8 and at most 256, the fine
// fields 16-byte aligned, the coarse field 16-byte aligned for the tensor map.
bool prolong_tma(float* x, const float* xc, const float* mask, int nx, int ny, int nz, int cx, int cy, int cz,
                 float alpha, cudaStream_t st) {
    if (nz % 8 != 0 || nz < 16 || nz > 256) return false;
    if ((reinterpret_cast<uintptr_t>(x) | reinterpret_cast<uintptr_t>(mask) | reinterpret_cast<uintptr_t>(xc)) & 15)
        return false;
    const EncodeTiled enc = encode_tiled();
    if (!enc) return false;
    const int R = 2 * (256 / nz > 1 ? 256 / nz : 1);
    const int rows = R / 2 + 2;
    CUtensorMap tm;
    const cuuint64_t dims[3] = {(cuuint64_t)cz, (cuuint64_t)cy, (cuuint64_t)cx};
    const cuuint64_t strides[2] = {(cuuint64_t)cz * 4, (cuuint64_t)cy * cz * 4};
    const cuuint32_t box[3] = {(cuuint32_t)cz, (cuuint32_t)rows, 2};
    const cuuint32_t es[3] = {1, 1, 1};
    if (enc(&tm, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, const_cast<float*>(xc), dims, strides, box, es,
            CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
            CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
        return false;
    const size_t smem = (size_t)2 * rows * cz * sizeof(float) + 8;   // tile + mbarrier
    const dim3 grid((unsigned)((ny + R - 1) / R), (unsigned)nx);
    k_prolong_tma<<<grid, PT_THREADS, smem, st>>>(tm, x, xc, mask, nx, ny, nz, cx, cy, cz, R, alpha);
    return true;
}
}  // namespace

extern "C" {

int fc_mg_prolong_correct(float* x, const float* x_coarse, const float* mask, int nx, int ny, int nz, int cx,
                          int cy, int cz, float alpha, void* stream) {
    if (!x || !x_coarse || !mask || nx < 1 || ny < 1 || nz < 1 || cx < 1 || cy < 1 || cz < 1) return FC_ERR_ARG;
    if ((long long)nx * ny * nz >= (1LL << 31)) return FC_ERR_ARG;
    if (nx == 2 * cx && ny == 2 * cy && nz == 2 * cz) {
        const Lvl g{nx, ny, nz, 0, 0};
        if (prolong_tma(x, x_coarse, mask, nx, ny, nz, cx, cy, cz, alpha, (cudaStream_t)stream)) {
            // the TMA-staged kernel took it
        } else if (nz >= 4 * PAIR_X && nz % 4 == 0 && pair_ok(g, {x, mask}) &&
            !((reinterpret_cast<uintptr_t>(x) | reinterpret_cast<uintptr_t>(mask)) & 15)) {
            // whole warps of four cells per thread on the wide levels
            const dim3 grid((unsigned)((nz + 4 * PAIR_X - 1) / (4 * PAIR_X)), (unsigned)((ny + PAIR_Y - 1) / PAIR_Y),
                            (unsigned)nx);
            k_prolong4<<<grid, dim3(PAIR_X, PAIR_Y), 0, (cudaStream_t)stream>>>(x, x_coarse, mask, nx, ny, nz, cx, cy,
                                                                              cz, alpha);
        } else if (pair_ok(g, {x, mask})) {
            k_prolong2<<<pair_grid(g), dim3(PAIR_X, PAIR_Y), 0, (cudaStream_t)stream>>>(x, x_coarse, mask, nx, ny, nz,
                                                                                       cx, cy, cz, alpha);
        } else {
            const dim3 grid((unsigned)((nz + 63) / 64), (unsigned)((ny + 3) / 4), (unsigned)nx);
            k_prolong_2to1<<<grid, BLOCK, 0, (cudaStream_t)stream>>>(x, x_coarse, mask, nx, ny, nz, cx, cy, cz,
                                                                      alpha);
        }
    } else {
        k_prolong_correct<<<grid_for((long long)nx * ny * nz), BLOCK, 0, (cudaStream_t)stream>>>(
            x, x_coarse, mask, nx, ny, nz, cx, cy, cz, alpha);
    }
    return launch_status();
}

long long fc_mg_reduce_workspace_bytes(long long n) {
    if (n < 0) return -1;
    return (long long)(grid_for(n) + 1) * (long long)sizeof(double);
}

int fc_mg_residual_norm2(const float* x, const float* b, const float* mask, const float* aE, const float* aW,
                         const float* aN, const float* aS, const float* aU, const float* aD, const float* diagL,
                         float dt, int nx, int ny, int nz, int ax, int out_idx, float* r_out, void* workspace,
                         long long workspace_bytes, double* result, void* stream) {
    Lvl g{nx, ny, nz, ax, out_idx};
    const long long n = (long long)nx * ny * nz;
    if (level_ok(g) || !x || !b || !workspace || !result) return FC_ERR_ARG;
    if (workspace_bytes < fc_mg_reduce_workspace_bytes(n)) return FC_ERR_ARG;
    Coef a{aE, aW, aN, aS, aU, aD, diagL};
    double* part = reinterpret_cast<double*>(workspace);
    const unsigned nb = grid_for(n);
    cudaStream_t st = (cudaStream_t)stream;
    k_residual_sq<<<nb, BLOCK, 0, st>>>(x, b, mask, a, dt, g, r_out, part);
    int rc = launch_status();
    if (rc) return rc;
    k_sum_partials<<<1, BLOCK, 0, st>>>(part, (int)nb, result);
    return launch_status();
}

long long fc_mg_heat_balance_workspace_bytes(long long n) {
    if (n < 0) return -1;
    return (long long)(grid_for(n) + 1) * 3 * (long long)sizeof(double);
}

int fc_mg_heat_balance(const float* T, const float* src, const float* mask, const float* aE, const float* aW,
                       const float* aN, const float* aS, const float* aU, const float* aD, const float* diagL, int nx,
                       int ny, int nz, int ax, int out_idx, void* workspace, long long workspace_bytes,
                       double* result3, void* stream) {
    Lvl g{nx, ny, nz, ax, out_idx};
    const long long n = (long long)nx * ny * nz;
    if (level_ok(g) || !T || !mask || !workspace || !result3 || !aE || !aW || !aN || !aS || !aU || !aD || !diagL)
        return FC_ERR_ARG;
    if (workspace_bytes < fc_mg_heat_balance_workspace_bytes(n)) return FC_ERR_ARG;
    Coef a{aE, aW, aN, aS, aU, aD, diagL};
    double* part = reinterpret_cast<double*>(workspace);
    const unsigned nb = grid_for(n);
    cudaStream_t st = (cudaStream_t)stream;
    k_heat_balance<<<nb, BLOCK, 0, st>>>(T, src, mask, a, g, part);
    int rc = launch_status();
    if (rc) return rc;
    k_sum_partials3<<<1, BLOCK, 0, st>>>(part, (int)nb, result3);
    return launch_status();
}

int fc_mg_build_coeffs(const float* k, const float* rho_cp, const float* u, const float* v, const float* w, int nx,
                       int ny, int nz, int ax, int out_idx, float dx, float s, float* aE, float* aW, float* aN,
                       float* aS, float* aU, float* aD, float* diagL, void* stream) {
    Lvl g{nx, ny, nz, ax, out_idx};
    if (level_ok(g) || !k || !rho_cp || !u || !v || !w || !aE || !aW || !aN || !aS || !aU || !aD || !diagL)
        return FC_ERR_ARG;
    const float cd = (float)((double)s / ((double)dx * (double)dx));
    const float ca = (float)((double)s / (double)dx);
    k_build_coeffs<<<grid_for((long long)nx * ny * nz), BLOCK, 0, (cudaStream_t)stream>>>(
        k, rho_cp, u, v, w, g, cd, ca, aE, aW, aN, aS, aU, aD, diagL);
    return launch_status();
}

int fc_mg_restrict_mean(const float* src, int nx, int ny, int nz, float* dst, int as_mask, void* stream) {
    const int cx = nx / 2, cy = ny / 2, cz = nz / 2;
    if (!src || !dst || cx < 1 || cy < 1 || cz < 1) return FC_ERR_ARG;
    k_restrict_mean<<<grid_for((long long)cx * cy * cz), BLOCK, 0, (cudaStream_t)stream>>>(src, nx, ny, nz, dst, cx, cy,
                                                                                            cz, as_mask);
    return launch_status();
}

int fc_mg_inv_diag(const float* diagL, const float* mask, float* inv_diagM, float dt, float omega, long long n,
                   void* stream) {
    if (!diagL || !mask || !inv_diagM || n < 0) return FC_ERR_ARG;
    if (n == 0) return FC_OK;
    k_inv_diag<<<grid_for(n), BLOCK, 0, (cudaStream_t)stream>>>(diagL, mask, inv_diagM, dt, omega, n);
    return launch_status();
}

// FP64 exact solve of the coarsest level: the dense inverse (n*n doubles) plus two
// pivot row/column buffer pairs (4 n doubles) in one caller allocation.
long long fc_mg_coarse_dense_bytes(int nx, int ny, int nz) {
    const long long n = (long long)nx * ny * nz;
    if (nx < 1 || ny < 1 || nz < 1 || n > CD_MAX_CELLS) return -1;
    return (n * n + 4 * n) * (long long)sizeof(double);
}

int fc_mg_coarse_dense_build(const float* aE, const float* aW, const float* aN, const float* aS, const float* aU,
                             const float* aD, const float* diagL, const float* mask, float dt, int nx, int ny, int nz,
                             int ax, int out_idx, double* inv, long long inv_bytes, void* stream) {
    Lvl g{nx, ny, nz, ax, out_idx};
    if (level_ok(g) || !aE || !aW || !aN || !aS || !aU || !aD || !mask || !inv) return FC_ERR_ARG;
    (void)diagL;   // the flux-form diagonal is the sum of the couplings
    const long long need = fc_mg_coarse_dense_bytes(nx, ny, nz);
    if (need < 0) return FC_ERR_TOO_LARGE;
    if (inv_bytes < need || (reinterpret_cast<uintptr_t>(inv) & 7)) return FC_ERR_ARG;
    const int n = nx * ny * nz;
    cudaStream_t st = (cudaStream_t)stream;
    if (cudaMemsetAsync(inv, 0, sizeof(double) * (size_t)n * n, st) != cudaSuccess) return FC_ERR_LAUNCH;
    Coef a{aE, aW, aN, aS, aU, aD, diagL};
    k_cd_assemble<<<grid_for(n), BLOCK, 0, st>>>(a, mask, (double)dt, g, inv, n);
    int rc = launch_status();
    if (rc) return rc;
    double* buf = inv + (size_t)n * n;       // row0, col0, row1, col1
    k_cd_seed<<<grid_for(n), BLOCK, 0, st>>>(inv, n, buf, buf + n);
    rc = launch_status();
    if (rc) return rc;
    const dim3 grid((unsigned)((n + CD_TX - 1) / CD_TX), (unsigned)((n + CD_TY - 1) / CD_TY));
    for (int p = 0; p < n; ++p) {
        double* cur = buf + (size_t)(p & 1) * 2 * n;
        double* nxt = buf + (size_t)((p + 1) & 1) * 2 * n;
        k_cd_pivot<<<grid, dim3(CD_TX, CD_TY), 0, st>>>(inv, n, p, cur, cur + n, nxt, nxt + n);
        rc = launch_status();
        if (rc) return rc;
    }
    return FC_OK;
}

int fc_mg_coarse_dense_apply(const double* inv, const float* b, const float* mask, float* x, int n, void* stream) {
    if (!inv || !b || !mask || !x || n < 1) return FC_ERR_ARG;
    if (n > CD_MAX_CELLS) return FC_ERR_TOO_LARGE;
    k_cd_apply<<<(unsigned)((n + 7) / 8), 256, sizeof(double) * (size_t)n, (cudaStream_t)stream>>>(inv, b, mask, x,
                                                                                                  n);
    return launch_status();
}

}  // extern "C"
