// fc_thermal.cu -- pseudo-time thermal step kernels (sm_103a) behind a C ABI.
//
// Reference: solver/thermal_kernels.cu (thermal_rhs :31-50, thermal_reconstruct
// :61-114, convergence_metrics + reduce_max :122-172, physics_check :180-189)
// and the steady residual of LBM_CHT.py:2690-2699.  Reductions here are
// two-pass per-block partials reduced by one block (max is order independent,
// so results are exact and deterministic); no process-global device state.
#include "fc_common.cuh"
#include "../../include/fluxcore3d_gb300.h"

using namespace fc;

namespace {

constexpr int BLOCK = 256;
inline unsigned grid_for(long long n) { return (unsigned)((n + BLOCK - 1) / BLOCK); }

__global__ void __launch_bounds__(BLOCK) k_rhs(const float* __restrict__ T_old, const float* __restrict__ T0,
                                               const float* __restrict__ src, const float* __restrict__ LT0,
                                               const float* __restrict__ mask, float* __restrict__ rhs,
                                               float* __restrict__ theta0, float dt, long long n) {
    const long long i = (long long)blockIdx.x * BLOCK + threadIdx.x;
    if (i >= n) return;
    const float m = mask[i], to = T_old[i];
    rhs[i] = m * ((to + dt * src[i]) - LT0[i]);
    theta0[i] = m * (to - T0[i]);
}

__global__ void __launch_bounds__(BLOCK) k_reconstruct(const float* __restrict__ T0, const float* __restrict__ th,
                                                       float* __restrict__ Tn, int nx, int ny, int nz, int ax,
                                                       int out_idx) {
    const long long idx = (long long)blockIdx.x * BLOCK + threadIdx.x;
    const long long nynz = (long long)ny * nz;
    if (idx >= nx * nynz) return;
    const int i = (int)(idx / nynz);
    const int r = (int)(idx - i * nynz);
    const int j = r / nz, k = r - (r / nz) * nz;
    long long s = idx;
    bool neu = false;
    // face priority x, then y, then z; high faces always Neumann, low faces unless
    // they are the inlet of the flow axis
    if (i == nx - 1) { neu = true; s = (i - 1) * nynz + (long long)j * nz + k; }
    else if (i == 0 && (ax != 0 || out_idx == 0)) { neu = true; s = 1 * nynz + (long long)j * nz + k; }
    if (!neu) {
        if (j == ny - 1) { neu = true; s = i * nynz + (long long)(j - 1) * nz + k; }
        else if (j == 0 && (ax != 1 || out_idx == 0)) { neu = true; s = i * nynz + (long long)1 * nz + k; }
    }
    if (!neu) {
        if (k == nz - 1) { neu = true; s = i * nynz + (long long)j * nz + (k - 1); }
        else if (k == 0 && (ax != 2 || out_idx == 0)) { neu = true; s = i * nynz + (long long)j * nz + 1; }
    }
    Tn[idx] = T0[s] + th[s];
}

// partial maxima of |T_new - T_old| over solid (slot 0) and fluid (slot 1) cells
__global__ void __launch_bounds__(BLOCK) k_dT_part(const float* __restrict__ Tn, const float* __restrict__ To,
                                                   const uint8_t* __restrict__ solid, float* __restrict__ part,
                                                   long long n) {
    __shared__ float ss[BLOCK], sf[BLOCK];
    float vs = 0.f, vf = 0.f;
    for (long long i = (long long)blockIdx.x * BLOCK + threadIdx.x; i < n; i += (long long)gridDim.x * BLOCK) {
        const float d = fabsf(Tn[i] - To[i]);
        if (solid[i]) vs = fmaxf(vs, d); else vf = fmaxf(vf, d);
    }
    ss[threadIdx.x] = vs;
    sf[threadIdx.x] = vf;
    __syncthreads();
    for (int s = BLOCK / 2; s > 0; s >>= 1) {
        if ((int)threadIdx.x < s) {
            ss[threadIdx.x] = fmaxf(ss[threadIdx.x], ss[threadIdx.x + s]);
            sf[threadIdx.x] = fmaxf(sf[threadIdx.x], sf[threadIdx.x + s]);
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) { part[2 * blockIdx.x] = ss[0]; part[2 * blockIdx.x + 1] = sf[0]; }
}

__global__ void __launch_bounds__(BLOCK) k_max2_final(const float* __restrict__ part, int nb, float* __restrict__ out) {
    __shared__ float a[BLOCK], b[BLOCK];
    float va = 0.f, vb = 0.f;
    for (int p = threadIdx.x; p < nb; p += BLOCK) { va = fmaxf(va, part[2 * p]); vb = fmaxf(vb, part[2 * p + 1]); }
    a[threadIdx.x] = va;
    b[threadIdx.x] = vb;
    __syncthreads();
    for (int s = BLOCK / 2; s > 0; s >>= 1) {
        if ((int)threadIdx.x < s) {
            a[threadIdx.x] = fmaxf(a[threadIdx.x], a[threadIdx.x + s]);
            b[threadIdx.x] = fmaxf(b[threadIdx.x], b[threadIdx.x + s]);
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) { out[0] = a[0]; out[1] = b[0]; }
}

__global__ void __launch_bounds__(BLOCK) k_physics(const float* __restrict__ T, int* __restrict__ flag, float tmin,
                                                   float tmax, long long n) {
    const long long i = (long long)blockIdx.x * BLOCK + threadIdx.x;
    if (i >= n) return;
    const float v = T[i];
    if (!isfinite(v) || v < tmin || v > tmax) atomicOr(flag, 1);
}

struct Lvl { int nx, ny, nz, ax, out_idx; };
__device__ __forceinline__ int lowg(const Lvl& g, int a) { return (g.ax == a && g.out_idx != 0) ? 0 : 1; }

// partial maxima of |mask (L T - src/dt)| (slot 0) and |src/dt| over mask (slot 1),
// L T evaluated as (M(T) - T)/dt like L_apply_fine
__global__ void __launch_bounds__(BLOCK) k_steady_part(const float* __restrict__ T, const float* __restrict__ aE,
                                                       const float* __restrict__ aW, const float* __restrict__ aN,
                                                       const float* __restrict__ aS, const float* __restrict__ aU,
                                                       const float* __restrict__ aD, const float* __restrict__ diagL,
                                                       const float* __restrict__ src, const float* __restrict__ mask,
                                                       float dt, Lvl g, float* __restrict__ part) {
    __shared__ float a[BLOCK], b[BLOCK];
    const long long n = (long long)g.nx * g.ny * g.nz;
    const long long nynz = (long long)g.ny * g.nz;
    float va = 0.f, vb = 0.f;
    for (long long idx = (long long)blockIdx.x * BLOCK + threadIdx.x; idx < n; idx += (long long)gridDim.x * BLOCK) {
        const int i = (int)(idx / nynz);
        const int rr = (int)(idx - i * nynz);
        const int j = rr / g.nz, k = rr - (rr / g.nz) * g.nz;
        const int iE = i < g.nx - 1 ? i + 1 : i - 1, iW = i > 0 ? i - 1 : lowg(g, 0);
        const int jN = j < g.ny - 1 ? j + 1 : j - 1, jS = j > 0 ? j - 1 : lowg(g, 1);
        const int kU = k < g.nz - 1 ? k + 1 : k - 1, kD = k > 0 ? k - 1 : lowg(g, 2);
        const float tc = T[idx];
        // flux form, as in the multigrid kernels (exact on constant fields)
        const float L = aE[idx] * (tc - T[iE * nynz + (long long)j * g.nz + k]) +
                        aW[idx] * (tc - T[iW * nynz + (long long)j * g.nz + k]) +
                        aN[idx] * (tc - T[i * nynz + (long long)jN * g.nz + k]) +
                        aS[idx] * (tc - T[i * nynz + (long long)jS * g.nz + k]) +
                        aU[idx] * (tc - T[i * nynz + (long long)j * g.nz + kU]) +
                        aD[idx] * (tc - T[i * nynz + (long long)j * g.nz + kD]);
        const float lo = tc + dt * L;
        const float LT = (lo - tc) / dt;
        const float ss = src[idx] / dt;
        const float m = mask[idx];
        va = fmaxf(va, fabsf((LT - ss) * m));
        if (m != 0.f) vb = fmaxf(vb, fabsf(ss));
    }
    a[threadIdx.x] = va;
    b[threadIdx.x] = vb;
    __syncthreads();
    for (int s = BLOCK / 2; s > 0; s >>= 1) {
        if ((int)threadIdx.x < s) {
            a[threadIdx.x] = fmaxf(a[threadIdx.x], a[threadIdx.x + s]);
            b[threadIdx.x] = fmaxf(b[threadIdx.x], b[threadIdx.x + s]);
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) { part[2 * blockIdx.x] = a[0]; part[2 * blockIdx.x + 1] = b[0]; }
}

constexpr int MAXB = 1184;
inline unsigned red_blocks(long long n) {
    const long long b = (n + BLOCK - 1) / BLOCK;
    return (unsigned)(b < MAXB ? (b < 1 ? 1 : b) : MAXB);
}

}  // namespace

extern "C" {

/* replaces THERMAL_CUDA.thermal_rhs */
int fc_thermal_rhs(const float* T_old, const float* T0, const float* src_step, const float* LT0, const float* mask_f,
                   float* rhs, float* theta0, float dt, long long n, void* stream) {
    if (!T_old || !T0 || !src_step || !LT0 || !mask_f || !rhs || !theta0 || n < 0) return FC_ERR_ARG;
    if (n == 0) return FC_OK;
    k_rhs<<<grid_for(n), BLOCK, 0, (cudaStream_t)stream>>>(T_old, T0, src_step, LT0, mask_f, rhs, theta0, dt, n);
    return launch_status();
}

int fc_thermal_reconstruct(const float* T0, const float* theta, float* T_new, int nx, int ny, int nz, int ax,
                           int out_idx, void* stream) {
    if (!T0 || !theta || !T_new || nx < 2 || ny < 2 || nz < 2 || ax < 0 || ax > 2) return FC_ERR_ARG;
    if (T_new == T0 || T_new == theta) return FC_ERR_ARG;
    k_reconstruct<<<grid_for((long long)nx * ny * nz), BLOCK, 0, (cudaStream_t)stream>>>(T0, theta, T_new, nx, ny, nz,
                                                                                          ax, out_idx);
    return launch_status();
}

long long fc_thermal_workspace_bytes(long long n) {
    if (n < 0) return -1;
    return (long long)red_blocks(n) * 2 * (long long)sizeof(float) + 16;
}

/* result: 2 device floats (max |dT| over solid, over fluid) */
int fc_thermal_convergence_metrics(const float* T_new, const float* T_old, const uint8_t* solid, long long n,
                                   void* workspace, long long workspace_bytes, float* result, void* stream) {
    if (!T_new || !T_old || !solid || !workspace || !result || n < 0) return FC_ERR_ARG;
    if (workspace_bytes < fc_thermal_workspace_bytes(n)) return FC_ERR_ARG;
    const unsigned nb = red_blocks(n);
    cudaStream_t st = (cudaStream_t)stream;
    k_dT_part<<<nb, BLOCK, 0, st>>>(T_new, T_old, solid, (float*)workspace, n);
    int rc = launch_status();
    if (rc) return rc;
    k_max2_final<<<1, BLOCK, 0, st>>>((const float*)workspace, (int)nb, result);
    return launch_status();
}

/* flag (device int32) |= 1 where T is non-finite or outside [T_min, T_max]; caller zeroes flag */
int fc_thermal_physics_check(const float* T, int* flag, float T_min, float T_max, long long n, void* stream) {
    if (!T || !flag || n < 0) return FC_ERR_ARG;
    if (n == 0) return FC_OK;
    k_physics<<<grid_for(n), BLOCK, 0, (cudaStream_t)stream>>>(T, flag, T_min, T_max, n);
    return launch_status();
}

/* result: 2 device floats (max |mask (L T - src/dt)|, max over mask of |src/dt|) */
int fc_thermal_steady_residual(const float* T, const float* aE, const float* aW, const float* aN, const float* aS,
                               const float* aU, const float* aD, const float* diagL, const float* src_step,
                               const float* mask, float dt, int nx, int ny, int nz, int ax, int out_idx,
                               void* workspace, long long workspace_bytes, float* result, void* stream) {
    const long long n = (long long)nx * ny * nz;
    if (!T || !src_step || !mask || !workspace || !result || nx < 2 || ny < 2 || nz < 2 || dt == 0.f)
        return FC_ERR_ARG;
    if (workspace_bytes < fc_thermal_workspace_bytes(n)) return FC_ERR_ARG;
    Lvl g{nx, ny, nz, ax, out_idx};
    const unsigned nb = red_blocks(n);
    cudaStream_t st = (cudaStream_t)stream;
    k_steady_part<<<nb, BLOCK, 0, st>>>(T, aE, aW, aN, aS, aU, aD, diagL, src_step, mask, dt, g, (float*)workspace);
    int rc = launch_status();
    if (rc) return rc;
    k_max2_final<<<1, BLOCK, 0, st>>>((const float*)workspace, (int)nb, result);
    return launch_status();
}

}  // extern "C"
