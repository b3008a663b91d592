// fc_krylov.cu -- vector kernels for the multigrid-preconditioned Krylov
// thermal solvers (sm_103a), behind a C ABI.
//
// Dot products and norms accumulate in FP64 with a fixed reduction order
// (per-block tree, then one block over the partials), so results are
// deterministic run to run.  Coefficients of updates can be read from device
// scalars so a Krylov iteration needs no host round trip except for its
// convergence test.  The FP64 operator apply M(x) = x + dt L(x) reads the
// FP32 7-point coefficients of the multigrid fine level and promotes them.
#include "fc_common.cuh"
#include "../../include/fluxcore3d_gb300.h"

#include <type_traits>

using namespace fc;

namespace {

constexpr int BLOCK = 256;
constexpr int MAX_BLOCKS = 1184;  // 152 SMs x 8 resident 256-thread blocks
inline unsigned grid_for(long long n) { return (unsigned)((n + BLOCK - 1) / BLOCK); }
inline unsigned red_blocks(long long n) {
    const long long b = (n + BLOCK - 1) / BLOCK;
    return (unsigned)(b < MAX_BLOCKS ? (b < 1 ? 1 : b) : MAX_BLOCKS);
}

// Each thread's strided partial sum is kept in FP32 when both vectors are FP32
// (a dozen terms per thread at the sizes used; promoting every element to FP64
// would cost more than the memory traffic on this part), in FP64 otherwise;
// partials are combined in FP64 in a fixed order.
template <typename A, typename B>
__global__ void __launch_bounds__(BLOCK) k_dot_part(const A* __restrict__ x, const B* __restrict__ y, long long n,
                                                    const float* __restrict__ w, double* __restrict__ part) {
    __shared__ double sh[BLOCK];
    constexpr bool F32 = sizeof(A) == 4 && sizeof(B) == 4;
    using Acc = typename std::conditional<F32, float, double>::type;
    Acc s = 0;
    for (long long i = (long long)blockIdx.x * BLOCK + threadIdx.x; i < n; i += (long long)gridDim.x * BLOCK) {
        Acc t = (Acc)x[i] * (Acc)y[i];
        if (w) t *= (Acc)w[i];
        s += t;
    }
    sh[threadIdx.x] = (double)s;
    __syncthreads();
    for (int st = BLOCK / 2; st > 0; st >>= 1) {
        if ((int)threadIdx.x < st) sh[threadIdx.x] += sh[threadIdx.x + st];
        __syncthreads();
    }
    if (threadIdx.x == 0) part[blockIdx.x] = sh[0];
}

__global__ void __launch_bounds__(BLOCK) k_sum(const double* __restrict__ part, int n, double* __restrict__ out) {
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

// y = alpha * x + beta * y, alpha = ha * (*da_num / *da_den) when da_num is set, else ha
template <typename T>
__global__ void __launch_bounds__(BLOCK) k_axpby(T* __restrict__ y, const T* __restrict__ x, long long n, double ha,
                                                 const double* __restrict__ da_num, const double* __restrict__ da_den,
                                                 double hb, const float* __restrict__ mask) {
    const long long i = (long long)blockIdx.x * BLOCK + threadIdx.x;
    if (i >= n) return;
    double a = ha;
    if (da_num) a *= *da_num / (da_den ? *da_den : 1.0);
    double r = a * (double)x[i];
    if (hb != 0.0) r += hb * (double)y[i];   // beta 0: y is not read (it may be uninitialised)
    if (mask && mask[i] == 0.f) r = 0.0;
    y[i] = (T)r;
}

// (the mask holds 0 / 1, so it selects; scale 1 skips the multiply: FP64 operations
// per element are expensive on this part)
template <typename S, typename D, bool SCALED>
__global__ void __launch_bounds__(BLOCK) k_convert(D* __restrict__ d, const S* __restrict__ s, long long n,
                                                   const float* __restrict__ mask, double scale) {
    const long long i = (long long)blockIdx.x * BLOCK + threadIdx.x;
    if (i >= n) return;
    D v;
    if (SCALED) v = (D)((double)s[i] * scale);
    else v = (D)s[i];
    if (mask && mask[i] == 0.f) v = (D)0;
    d[i] = v;
}

struct Lvl { int nx, ny, nz, ax, out_idx; };
__device__ __forceinline__ int lowg(const Lvl& g, int a) { return (g.ax == a && g.out_idx != 0) ? 0 : 1; }

// y = M(x) = x + dt L(x) in the vectors' precision T (optionally masked, optionally r = b - M(x))
template <typename T>
__global__ void __launch_bounds__(BLOCK) k_mop_t(const T* __restrict__ x, const float* __restrict__ aE,
                                                   const float* __restrict__ aW, const float* __restrict__ aN,
                                                   const float* __restrict__ aS, const float* __restrict__ aU,
                                                   const float* __restrict__ aD, const float* __restrict__ diagL,
                                                   T dt, Lvl g, const T* __restrict__ b,
                                                   const float* __restrict__ mask, T* __restrict__ y) {
    const long long n = (long long)g.nx * g.ny * g.nz;
    const long long idx = (long long)blockIdx.x * BLOCK + threadIdx.x;
    if (idx >= n) return;
    const long long nynz = (long long)g.ny * g.nz;
    const int i = (int)idx / (int)nynz;
    const int rr = (int)idx - i * (int)nynz;
    const int j = rr / g.nz, k = rr - j * g.nz;
    const int iE = i < g.nx - 1 ? i + 1 : i - 1, iW = i > 0 ? i - 1 : lowg(g, 0);
    const int jN = j < g.ny - 1 ? j + 1 : j - 1, jS = j > 0 ? j - 1 : lowg(g, 1);
    const int kU = k < g.nz - 1 ? k + 1 : k - 1, kD = k > 0 ? k - 1 : lowg(g, 2);
    const T xc = x[idx];
    // flux form sum_n a_n (x_c - x_n): exact on constant fields (diagL = sum_n a_n is
    // not, once rounded to FP32), as in the multigrid kernels
    const T L = (T)aE[idx] * (xc - x[iE * nynz + (long long)j * g.nz + k]) +
                (T)aW[idx] * (xc - x[iW * nynz + (long long)j * g.nz + k]) +
                (T)aN[idx] * (xc - x[i * nynz + (long long)jN * g.nz + k]) +
                (T)aS[idx] * (xc - x[i * nynz + (long long)jS * g.nz + k]) +
                (T)aU[idx] * (xc - x[i * nynz + (long long)j * g.nz + kU]) +
                (T)aD[idx] * (xc - x[i * nynz + (long long)j * g.nz + kD]);
    T m = xc + dt * L;
    if (b) m = b[idx] - m;
    if (mask && mask[idx] == 0.f) m = (T)0;
    y[idx] = m;
}

// ---- BiCGSTAB recurrences with device scalars (slot layout in the header) ----
// The scalars are formed once by a one-thread kernel, so vector kernels never
// divide (FP64 division per element would dominate: GB300's FP64 rate is low).
enum BicgSlot { SL_RHO_NEW = 0, SL_RHO_OLD = 1, SL_ALPHA = 2, SL_OMEGA = 3, SL_RV = 4, SL_TS = 5, SL_TT = 6,
                SL_RR = 7, SL_BETA = 8 };

// stage 0: beta = (rho_new / rho_old) (alpha / omega) (0 when undefined)
// stage 1: alpha = rho_new / (r_hat, v)
// stage 2: omega = (t, s) / (t, t), rho_old = rho_new
__global__ void k_bicg_scalars(double* __restrict__ sc, int stage) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    if (stage == 0) {
        const double ro = sc[SL_RHO_OLD], om = sc[SL_OMEGA];
        sc[SL_BETA] = (ro != 0.0 && om != 0.0) ? (sc[SL_RHO_NEW] / ro) * (sc[SL_ALPHA] / om) : 0.0;
    } else if (stage == 1) {
        const double rv = sc[SL_RV];
        sc[SL_ALPHA] = rv != 0.0 ? sc[SL_RHO_NEW] / rv : 0.0;
    } else {
        const double tt = sc[SL_TT];
        sc[SL_OMEGA] = tt > 0.0 ? sc[SL_TS] / tt : 0.0;
        sc[SL_RHO_OLD] = sc[SL_RHO_NEW];
    }
}

// p = r + beta (p - omega v)
template <typename T>
__global__ void __launch_bounds__(BLOCK) k_bicg_p(T* __restrict__ p, const T* __restrict__ r,
                                                  const T* __restrict__ v, long long n,
                                                  const double* __restrict__ sc) {
    const long long i = (long long)blockIdx.x * BLOCK + threadIdx.x;
    if (i >= n) return;
    const T beta = (T)sc[SL_BETA], om = (T)sc[SL_OMEGA];
    const T p1 = -om * v[i] + p[i];
    p[i] = r[i] + beta * p1;
}

// stage 0: r -= alpha w; x += alpha u
// stage 1: x += omega u; r -= omega w; part = per-block (r, r) in FP64
template <typename T>
__global__ void __launch_bounds__(BLOCK) k_bicg_xr(T* __restrict__ x, T* __restrict__ r, const T* __restrict__ u,
                                                   const T* __restrict__ w, long long n,
                                                   const double* __restrict__ sc, int stage,
                                                   double* __restrict__ part) {
    __shared__ double sh[BLOCK];
    const T a = (T)sc[stage == 0 ? SL_ALPHA : SL_OMEGA];
    T s = 0;
    for (long long i = (long long)blockIdx.x * BLOCK + threadIdx.x; i < n; i += (long long)gridDim.x * BLOCK) {
        const T ri = -a * w[i] + r[i];
        r[i] = ri;
        x[i] = a * u[i] + x[i];
        if (stage == 1) s += ri * ri;
    }
    if (stage == 1) {
        sh[threadIdx.x] = (double)s;
        __syncthreads();
        for (int st = BLOCK / 2; st > 0; st >>= 1) {
            if ((int)threadIdx.x < st) sh[threadIdx.x] += sh[threadIdx.x + st];
            __syncthreads();
        }
        if (threadIdx.x == 0) part[blockIdx.x] = sh[0];
    }
}

// (x, y1) and (x, y2) in one pass, FP64 accumulation: partials [0, nb) and [nb, 2 nb)
template <typename T>
__global__ void __launch_bounds__(BLOCK) k_dot2_part(const T* __restrict__ x, const T* __restrict__ y1,
                                                     const T* __restrict__ y2, long long n,
                                                     double* __restrict__ part) {
    __shared__ double sa[BLOCK], sb[BLOCK];
    T a = 0, b = 0;   // per-thread partials in the vectors' precision (as k_dot_part)
    for (long long i = (long long)blockIdx.x * BLOCK + threadIdx.x; i < n; i += (long long)gridDim.x * BLOCK) {
        const T xi = x[i];
        a += xi * y1[i];
        b += xi * y2[i];
    }
    sa[threadIdx.x] = (double)a;
    sb[threadIdx.x] = (double)b;
    __syncthreads();
    for (int st = BLOCK / 2; st > 0; st >>= 1) {
        if ((int)threadIdx.x < st) {
            sa[threadIdx.x] += sa[threadIdx.x + st];
            sb[threadIdx.x] += sb[threadIdx.x + st];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        part[blockIdx.x] = sa[0];
        part[gridDim.x + blockIdx.x] = sb[0];
    }
}

// y += M^T (mask * x), scattered: row r of M holds 1 + dt sum_n a_n(r) on the diagonal and
// -dt a_n(r) at its (ghosted) neighbour n, so row r adds x_r times each entry to the column
// it sits in.  A ghost that maps a direction onto the cell itself adds +dt a_n and -dt a_n to
// the same column, as the row does.  y must be zero on entry.
__global__ void __launch_bounds__(BLOCK) k_mop_transpose(const float* __restrict__ x, const float* __restrict__ aE,
                                                         const float* __restrict__ aW, const float* __restrict__ aN,
                                                         const float* __restrict__ aS, const float* __restrict__ aU,
                                                         const float* __restrict__ aD, float dt, Lvl g,
                                                         const float* __restrict__ mask, float* __restrict__ y) {
    const long long n = (long long)g.nx * g.ny * g.nz;
    const long long idx = (long long)blockIdx.x * BLOCK + threadIdx.x;
    if (idx >= n) return;
    if (mask && mask[idx] == 0.f) return;
    const float v = x[idx];
    if (v == 0.f) return;
    const long long nynz = (long long)g.ny * g.nz;
    const int i = (int)idx / (int)nynz;
    const int rr = (int)idx - i * (int)nynz;
    const int j = rr / g.nz, k = rr - j * g.nz;
    const int iE = i < g.nx - 1 ? i + 1 : i - 1, iW = i > 0 ? i - 1 : lowg(g, 0);
    const int jN = j < g.ny - 1 ? j + 1 : j - 1, jS = j > 0 ? j - 1 : lowg(g, 1);
    const int kU = k < g.nz - 1 ? k + 1 : k - 1, kD = k > 0 ? k - 1 : lowg(g, 2);
    const float e = aE[idx], w = aW[idx], nn = aN[idx], s = aS[idx], u = aU[idx], d = aD[idx];
    const float dv = dt * v;
    atomicAdd(y + idx, v + dv * (((e + w) + (nn + s)) + (u + d)));
    atomicAdd(y + iE * nynz + (long long)j * g.nz + k, -dv * e);
    atomicAdd(y + iW * nynz + (long long)j * g.nz + k, -dv * w);
    atomicAdd(y + i * nynz + (long long)jN * g.nz + k, -dv * nn);
    atomicAdd(y + i * nynz + (long long)jS * g.nz + k, -dv * s);
    atomicAdd(y + i * nynz + (long long)j * g.nz + kU, -dv * u);
    atomicAdd(y + i * nynz + (long long)j * g.nz + kD, -dv * d);
}

}  // namespace

extern "C" {

long long fc_vec_workspace_bytes(long long n) {
    if (n < 0) return -1;
    return (long long)(red_blocks(n) + 1) * (long long)sizeof(double);
}

// kind: 0 = (f64, f64), 1 = (f32, f32), 2 = (f64, f32).  result: device double.
int fc_vec_dot(int kind, const void* x, const void* y, long long n, const float* weight, void* workspace,
               long long workspace_bytes, double* result, void* stream) {
    if (!x || !y || !result || !workspace || n < 0) return FC_ERR_ARG;
    if (workspace_bytes < fc_vec_workspace_bytes(n)) return FC_ERR_ARG;
    const unsigned nb = red_blocks(n);
    double* part = reinterpret_cast<double*>(workspace);
    cudaStream_t st = (cudaStream_t)stream;
    switch (kind) {
        case 0: k_dot_part<double, double><<<nb, BLOCK, 0, st>>>((const double*)x, (const double*)y, n, weight, part); break;
        case 1: k_dot_part<float, float><<<nb, BLOCK, 0, st>>>((const float*)x, (const float*)y, n, weight, part); break;
        case 2: k_dot_part<double, float><<<nb, BLOCK, 0, st>>>((const double*)x, (const float*)y, n, weight, part); break;
        default: return FC_ERR_ARG;
    }
    int rc = launch_status();
    if (rc) return rc;
    k_sum<<<1, BLOCK, 0, st>>>(part, (int)nb, result);
    return launch_status();
}

// y = alpha x + beta y ; alpha = alpha_host * (*alpha_num / *alpha_den) when alpha_num != NULL
int fc_vec_axpby(int is_f64, void* y, const void* x, long long n, double alpha_host, const double* alpha_num,
                 const double* alpha_den, double beta, const float* mask, void* stream) {
    if (!y || !x || n < 0) return FC_ERR_ARG;
    if (n == 0) return FC_OK;
    cudaStream_t st = (cudaStream_t)stream;
    if (is_f64)
        k_axpby<double><<<grid_for(n), BLOCK, 0, st>>>((double*)y, (const double*)x, n, alpha_host, alpha_num, alpha_den, beta, mask);
    else
        k_axpby<float><<<grid_for(n), BLOCK, 0, st>>>((float*)y, (const float*)x, n, alpha_host, alpha_num, alpha_den, beta, mask);
    return launch_status();
}

// dst = scale * src (* mask); kind 0 f32->f64, 1 f64->f32, 2 f32->f32, 3 f64->f64
int fc_vec_convert(int kind, void* dst, const void* src, long long n, const float* mask, double scale, void* stream) {
    if (!dst || !src || n < 0) return FC_ERR_ARG;
    if (n == 0) return FC_OK;
    cudaStream_t st = (cudaStream_t)stream;
    const unsigned g = grid_for(n);
#define FC_CONV(K, S, D)                                                                                     \
    case K:                                                                                                 \
        if (scale == 1.0) k_convert<S, D, false><<<g, BLOCK, 0, st>>>((D*)dst, (const S*)src, n, mask, scale); \
        else k_convert<S, D, true><<<g, BLOCK, 0, st>>>((D*)dst, (const S*)src, n, mask, scale);              \
        break;
    switch (kind) {
        FC_CONV(0, float, double)
        FC_CONV(1, double, float)
        FC_CONV(2, float, float)
        FC_CONV(3, double, double)
        default: return FC_ERR_ARG;
    }
#undef FC_CONV
    return launch_status();
}

long long fc_vec_dot2_workspace_bytes(long long n) {
    if (n < 0) return -1;
    return (long long)(2 * red_blocks(n) + 2) * (long long)sizeof(double);
}

int fc_vec_dot2(int is_f64, const void* x, const void* y1, const void* y2, long long n, void* workspace,
                long long workspace_bytes, double* result2, void* stream) {
    if (!x || !y1 || !y2 || !result2 || !workspace || n < 0) return FC_ERR_ARG;
    if (workspace_bytes < fc_vec_dot2_workspace_bytes(n)) return FC_ERR_ARG;
    const unsigned nb = red_blocks(n);
    double* part = reinterpret_cast<double*>(workspace);
    cudaStream_t st = (cudaStream_t)stream;
    if (is_f64)
        k_dot2_part<double><<<nb, BLOCK, 0, st>>>((const double*)x, (const double*)y1, (const double*)y2, n, part);
    else
        k_dot2_part<float><<<nb, BLOCK, 0, st>>>((const float*)x, (const float*)y1, (const float*)y2, n, part);
    int rc = launch_status();
    if (rc) return rc;
    k_sum<<<1, BLOCK, 0, st>>>(part, (int)nb, result2);
    rc = launch_status();
    if (rc) return rc;
    k_sum<<<1, BLOCK, 0, st>>>(part + nb, (int)nb, result2 + 1);
    return launch_status();
}

int fc_bicgstab_p(int is_f64, void* p, const void* r, const void* v, long long n, double* scalars, void* stream) {
    if (!p || !r || !v || !scalars || n < 0) return FC_ERR_ARG;
    cudaStream_t st = (cudaStream_t)stream;
    k_bicg_scalars<<<1, 32, 0, st>>>(scalars, 0);
    int rc = launch_status();
    if (rc || n == 0) return rc;
    if (is_f64)
        k_bicg_p<double><<<grid_for(n), BLOCK, 0, st>>>((double*)p, (const double*)r, (const double*)v, n, scalars);
    else
        k_bicg_p<float><<<grid_for(n), BLOCK, 0, st>>>((float*)p, (const float*)r, (const float*)v, n, scalars);
    return launch_status();
}

int fc_bicgstab_xr(int is_f64, void* x, void* r, const void* u, const void* w, long long n, double* scalars,
                   int stage, void* workspace, long long workspace_bytes, void* stream) {
    if (!x || !r || !u || !w || !scalars || n < 0 || (stage != 0 && stage != 1)) return FC_ERR_ARG;
    if (stage == 1 && (!workspace || workspace_bytes < fc_vec_workspace_bytes(n))) return FC_ERR_ARG;
    cudaStream_t st = (cudaStream_t)stream;
    k_bicg_scalars<<<1, 32, 0, st>>>(scalars, stage == 0 ? 1 : 2);
    int rc = launch_status();
    if (rc) return rc;
    const unsigned nb = red_blocks(n);
    double* part = reinterpret_cast<double*>(workspace);
    if (is_f64)
        k_bicg_xr<double><<<nb, BLOCK, 0, st>>>((double*)x, (double*)r, (const double*)u, (const double*)w, n,
                                                scalars, stage, part);
    else
        k_bicg_xr<float><<<nb, BLOCK, 0, st>>>((float*)x, (float*)r, (const float*)u, (const float*)w, n, scalars,
                                               stage, part);
    rc = launch_status();
    if (rc) return rc;
    if (stage == 1) {
        k_sum<<<1, BLOCK, 0, st>>>(part, (int)nb, scalars + SL_RR);
        rc = launch_status();
    }
    return rc;
}

// y = M(x) (b == NULL) or y = b - M(x); optionally multiplied by mask.  FP64 vectors, FP32 coefficients.
int fc_mg_mop_f64(const double* x, const float* aE, const float* aW, const float* aN, const float* aS,
                  const float* aU, const float* aD, const float* diagL, double dt, int nx, int ny, int nz, int ax,
                  int out_idx, const double* b, const float* mask, double* y, void* stream) {
    if (!x || !y || !aE || !aW || !aN || !aS || !aU || !aD || !diagL || nx < 2 || ny < 2 || nz < 2 || ax < 0 || ax > 2)
        return FC_ERR_ARG;
    if (x == y || (long long)nx * ny * nz >= (1LL << 31)) return FC_ERR_ARG;
    Lvl g{nx, ny, nz, ax, out_idx};
    k_mop_t<double><<<grid_for((long long)nx * ny * nz), BLOCK, 0, (cudaStream_t)stream>>>(
        x, aE, aW, aN, aS, aU, aD, diagL, dt, g, b, mask, y);
    return launch_status();
}

int fc_mg_mop_transpose_f32(const float* x, const float* aE, const float* aW, const float* aN, const float* aS,
                            const float* aU, const float* aD, float dt, int nx, int ny, int nz, int ax,
                            int out_idx, const float* mask, float* y, void* stream) {
    if (!x || !y || !aE || !aW || !aN || !aS || !aU || !aD || nx < 2 || ny < 2 || nz < 2 || ax < 0 || ax > 2)
        return FC_ERR_ARG;
    if (x == y || (long long)nx * ny * nz >= (1LL << 31)) return FC_ERR_ARG;
    const long long n = (long long)nx * ny * nz;
    cudaStream_t st = (cudaStream_t)stream;
    if (cudaMemsetAsync(y, 0, (size_t)n * sizeof(float), st) != cudaSuccess) return FC_ERR_LAUNCH;
    Lvl g{nx, ny, nz, ax, out_idx};
    k_mop_transpose<<<grid_for(n), BLOCK, 0, st>>>(x, aE, aW, aN, aS, aU, aD, dt, g, mask, y);
    return launch_status();
}

// The same operator on FP32 vectors (the inner solve of the mixed-precision solver).
int fc_mg_mop_f32(const float* x, const float* aE, const float* aW, const float* aN, const float* aS,
                  const float* aU, const float* aD, const float* diagL, float dt, int nx, int ny, int nz, int ax,
                  int out_idx, const float* b, const float* mask, float* y, void* stream) {
    if (!x || !y || !aE || !aW || !aN || !aS || !aU || !aD || !diagL || nx < 2 || ny < 2 || nz < 2 || ax < 0 || ax > 2)
        return FC_ERR_ARG;
    if (x == y || (long long)nx * ny * nz >= (1LL << 31)) return FC_ERR_ARG;
    Lvl g{nx, ny, nz, ax, out_idx};
    k_mop_t<float><<<grid_for((long long)nx * ny * nz), BLOCK, 0, (cudaStream_t)stream>>>(
        x, aE, aW, aN, aS, aU, aD, diagL, dt, g, b, mask, y);
    return launch_status();
}

}  // extern "C"
