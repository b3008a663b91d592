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

using namespace fc;

namespace {

constexpr int BLOCK = 256;
constexpr int MAX_BLOCKS = 1184;  // 152 SMs x 8 resident 256-thread blocks
inline unsigned grid_for(long long n) { return (unsigned)((n + BLOCK - 1) / BLOCK); }
inline unsigned red_blocks(long long n) {
    const long long b = (n + BLOCK - 1) / BLOCK;
    return (unsigned)(b < MAX_BLOCKS ? (b < 1 ? 1 : b) : MAX_BLOCKS);
}

template <typename A, typename B>
__global__ void __launch_bounds__(BLOCK) k_dot_part(const A* __restrict__ x, const B* __restrict__ y, long long n,
                                                    const float* __restrict__ w, double* __restrict__ part) {
    __shared__ double sh[BLOCK];
    double s = 0.0;
    for (long long i = (long long)blockIdx.x * BLOCK + threadIdx.x; i < n; i += (long long)gridDim.x * BLOCK) {
        double t = (double)x[i] * (double)y[i];
        if (w) t *= (double)w[i];
        s += t;
    }
    sh[threadIdx.x] = s;
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
    double r = a * (double)x[i] + hb * (double)y[i];
    if (mask) r *= (double)mask[i];
    y[i] = (T)r;
}

template <typename S, typename D>
__global__ void __launch_bounds__(BLOCK) k_convert(D* __restrict__ d, const S* __restrict__ s, long long n,
                                                   const float* __restrict__ mask, double scale) {
    const long long i = (long long)blockIdx.x * BLOCK + threadIdx.x;
    if (i >= n) return;
    double v = (double)s[i] * scale;
    if (mask) v *= (double)mask[i];
    d[i] = (D)v;
}

struct Lvl { int nx, ny, nz, ax, out_idx; };
__device__ __forceinline__ int lowg(const Lvl& g, int a) { return (g.ax == a && g.out_idx != 0) ? 0 : 1; }

// y = M(x) = x + dt L(x) in FP64 (optionally masked, optionally r = b - M(x))
__global__ void __launch_bounds__(BLOCK) k_mop_f64(const double* __restrict__ x, const float* __restrict__ aE,
                                                   const float* __restrict__ aW, const float* __restrict__ aN,
                                                   const float* __restrict__ aS, const float* __restrict__ aU,
                                                   const float* __restrict__ aD, const float* __restrict__ diagL,
                                                   double dt, Lvl g, const double* __restrict__ b,
                                                   const float* __restrict__ mask, double* __restrict__ y) {
    const long long n = (long long)g.nx * g.ny * g.nz;
    const long long idx = (long long)blockIdx.x * BLOCK + threadIdx.x;
    if (idx >= n) return;
    const long long nynz = (long long)g.ny * g.nz;
    const int i = (int)(idx / nynz);
    const int rr = (int)(idx - i * nynz);
    const int j = rr / g.nz, k = rr - (rr / g.nz) * g.nz;
    const int iE = i < g.nx - 1 ? i + 1 : i - 1, iW = i > 0 ? i - 1 : lowg(g, 0);
    const int jN = j < g.ny - 1 ? j + 1 : j - 1, jS = j > 0 ? j - 1 : lowg(g, 1);
    const int kU = k < g.nz - 1 ? k + 1 : k - 1, kD = k > 0 ? k - 1 : lowg(g, 2);
    const double xc = x[idx];
    const double L = (double)diagL[idx] * xc - (double)aE[idx] * x[iE * nynz + (long long)j * g.nz + k] -
                     (double)aW[idx] * x[iW * nynz + (long long)j * g.nz + k] -
                     (double)aN[idx] * x[i * nynz + (long long)jN * g.nz + k] -
                     (double)aS[idx] * x[i * nynz + (long long)jS * g.nz + k] -
                     (double)aU[idx] * x[i * nynz + (long long)j * g.nz + kU] -
                     (double)aD[idx] * x[i * nynz + (long long)j * g.nz + kD];
    double m = xc + dt * L;
    if (b) m = b[idx] - m;
    if (mask) m *= (double)mask[idx];
    y[idx] = m;
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
    switch (kind) {
        case 0: k_convert<float, double><<<g, BLOCK, 0, st>>>((double*)dst, (const float*)src, n, mask, scale); break;
        case 1: k_convert<double, float><<<g, BLOCK, 0, st>>>((float*)dst, (const double*)src, n, mask, scale); break;
        case 2: k_convert<float, float><<<g, BLOCK, 0, st>>>((float*)dst, (const float*)src, n, mask, scale); break;
        case 3: k_convert<double, double><<<g, BLOCK, 0, st>>>((double*)dst, (const double*)src, n, mask, scale); break;
        default: return FC_ERR_ARG;
    }
    return launch_status();
}

// y = M(x) (b == NULL) or y = b - M(x); optionally multiplied by mask.  FP64 vectors, FP32 coefficients.
int fc_mg_mop_f64(const double* x, const float* aE, const float* aW, const float* aN, const float* aS,
                  const float* aU, const float* aD, const float* diagL, double dt, int nx, int ny, int nz, int ax,
                  int out_idx, const double* b, const float* mask, double* y, void* stream) {
    if (!x || !y || !aE || !aW || !aN || !aS || !aU || !aD || !diagL || nx < 2 || ny < 2 || nz < 2 || ax < 0 || ax > 2)
        return FC_ERR_ARG;
    if (x == y) return FC_ERR_ARG;
    Lvl g{nx, ny, nz, ax, out_idx};
    k_mop_f64<<<grid_for((long long)nx * ny * nz), BLOCK, 0, (cudaStream_t)stream>>>(x, aE, aW, aN, aS, aU, aD, diagL,
                                                                                      dt, g, b, mask, y);
    return launch_status();
}

}  // extern "C"
