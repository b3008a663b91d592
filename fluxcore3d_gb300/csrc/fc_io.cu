// fc_io.cu -- device side of snapshot and checkpoint I/O.
//
//  * fc_snapshot_pack: one frame of the reference's snapshot file
//    (LBMCHT3D_Torch._save_snapshot, LBM_CHT.py:2749-2769) packed into one
//    staging buffer in a single pass: the selected fields among u, v, w,
//    speed = sqrt(u*u + v*v + w*w), rho and T, each N floats, in that order.
//    speed is rounded as torch rounds its elementwise expression (u*u, v*v,
//    their sum, w*w, the sum, the square root; no contraction).  The caller
//    copies the staging buffer to pinned host memory on a copy stream, so
//    taking a snapshot costs the time loop one pass of 4-6 B in / out per field.
//  * fc_lbm_mass: the FP64 mass integral of a population buffer (sum of f over
//    the fluid cells), in a fixed-order two-stage reduction.
//  * fc_columns_gather / fc_columns_scatter: out[r][j] = src[r*ld + idx[j]] and
//    its inverse, for the populations of the inlet/outlet plane cells that a
//    checkpoint must carry (rows = 19 directions, ld = N).
#include "fc_common.cuh"
#include "../../include/fluxcore3d_gb300.h"

using namespace fc;

namespace {

constexpr int IO_BLOCK = 256;

enum SnapField : int { SF_U = 1, SF_V = 2, SF_W = 4, SF_SPEED = 8, SF_RHO = 16, SF_T = 32, SF_ALL = 63 };

struct PackArgs {
    const float* rho;
    const float* u;
    const float* v;
    const float* w;
    const float* T;
    float* out[6];   // destination of each field in output order (null: not selected)
    long long n;
};

__global__ void __launch_bounds__(IO_BLOCK) k_snapshot_pack(PackArgs a) {
    const long long stride = (long long)gridDim.x * IO_BLOCK;
    for (long long i = (long long)blockIdx.x * IO_BLOCK + threadIdx.x; i < a.n; i += stride) {
        const bool need_uvw = a.out[0] || a.out[1] || a.out[2] || a.out[3];
        float u = 0.f, v = 0.f, w = 0.f;
        if (need_uvw) {
            u = __ldg(a.u + i);
            v = __ldg(a.v + i);
            w = __ldg(a.w + i);
        }
        if (a.out[0]) a.out[0][i] = u;
        if (a.out[1]) a.out[1][i] = v;
        if (a.out[2]) a.out[2][i] = w;
        if (a.out[3]) a.out[3][i] = __fsqrt_rn(__fadd_rn(__fadd_rn(__fmul_rn(u, u), __fmul_rn(v, v)), __fmul_rn(w, w)));
        if (a.out[4]) a.out[4][i] = __ldg(a.rho + i);
        if (a.out[5]) a.out[5][i] = __ldg(a.T + i);
    }
}

template <bool SCATTER>
__global__ void __launch_bounds__(IO_BLOCK) k_columns(float* __restrict__ big, float* __restrict__ cols, int rows,
                                                      long long ld, const long long* __restrict__ idx, long long m,
                                                      unsigned* __restrict__ err) {
    const long long total = (long long)rows * m;
    const long long stride = (long long)gridDim.x * IO_BLOCK;
    for (long long t = (long long)blockIdx.x * IO_BLOCK + threadIdx.x; t < total; t += stride) {
        const long long r = t / m, j = t - r * m;
        const long long c = idx[j];
        if (c < 0 || c >= ld) {
            atomicOr(err, DEV_ERR_INDEX);
            continue;
        }
        if (SCATTER) big[r * ld + c] = cols[t];
        else cols[t] = big[r * ld + c];
    }
}

// a stored population as FP64 (shifted storage: the 16-bit deviation plus w_q, added in FP64)
template <int KIND, class T>
__device__ __forceinline__ double decode64(T v, int q) {
    if constexpr (KIND == ST_F32) return (double)v;
    else if constexpr (KIND == ST_F16S) return (double)__half2float(v) + (double)wq(q);
    else return (double)__bfloat162float(v) + (double)wq(q);
}

// FP64 mass integral: per-block sums over the cells with flag bit CF_SOLID clear of
// sum_q f_q (storage decoded: shifted storage adds w_q back)
template <int KIND>
__global__ void __launch_bounds__(IO_BLOCK) k_mass(const void* __restrict__ pop, const uint8_t* __restrict__ flags,
                                                   long long n, double* __restrict__ part) {
    __shared__ double sh[IO_BLOCK];
    using T = typename Store<KIND>::T;
    const T* p = reinterpret_cast<const T*>(pop);
    double v = 0.0;
    const long long stride = (long long)gridDim.x * IO_BLOCK;
    for (long long c = (long long)blockIdx.x * IO_BLOCK + threadIdx.x; c < n; c += stride) {
        if (flags && (flags[c] & CF_SOLID)) continue;
        double s = 0.0;
#pragma unroll
        for (int q = 0; q < 19; ++q) s += decode64<KIND>(p[(long long)q * n + c], q);
        v += s;
    }
    sh[threadIdx.x] = v;
    __syncthreads();
    for (int s = IO_BLOCK / 2; s > 0; s >>= 1) {
        if ((int)threadIdx.x < s) sh[threadIdx.x] += sh[threadIdx.x + s];
        __syncthreads();
    }
    if (threadIdx.x == 0) part[blockIdx.x] = sh[0];
}

__global__ void __launch_bounds__(IO_BLOCK) k_mass_sum(const double* __restrict__ part, int n,
                                                       double* __restrict__ out) {
    __shared__ double sh[IO_BLOCK];
    double v = 0.0;
    for (int p = threadIdx.x; p < n; p += IO_BLOCK) v += part[p];
    sh[threadIdx.x] = v;
    __syncthreads();
    for (int s = IO_BLOCK / 2; s > 0; s >>= 1) {
        if ((int)threadIdx.x < s) sh[threadIdx.x] += sh[threadIdx.x + s];
        __syncthreads();
    }
    if (threadIdx.x == 0) *out = sh[0];
}

constexpr int MASS_BLOCKS = 152 * 8;

unsigned grid_for(long long n) {
    long long b = (n + IO_BLOCK - 1) / IO_BLOCK;
    if (b > 152LL * 64) b = 152LL * 64;
    return (unsigned)(b < 1 ? 1 : b);
}

}  // namespace

extern "C" {

int fc_snapshot_pack(const float* rho, const float* u, const float* v, const float* w, const float* T, long long n,
                     int fields, float* out, void* stream) {
    if (n < 0 || !out || fields <= 0 || (fields & ~SF_ALL)) return FC_ERR_ARG;
    if ((fields & (SF_U | SF_V | SF_W | SF_SPEED)) && (!u || !v || !w)) return FC_ERR_ARG;
    if ((fields & SF_RHO) && !rho) return FC_ERR_ARG;
    if ((fields & SF_T) && !T) return FC_ERR_ARG;
    if (n == 0) return FC_OK;
    PackArgs a{rho, u, v, w, T, {nullptr, nullptr, nullptr, nullptr, nullptr, nullptr}, n};
    long long slot = 0;
    for (int f = 0; f < 6; ++f)
        if (fields & (1 << f)) a.out[f] = out + (slot++) * n;
    k_snapshot_pack<<<grid_for(n), IO_BLOCK, 0, (cudaStream_t)stream>>>(a);
    return launch_status();
}

int fc_columns_gather(const float* src, int rows, long long ld, const long long* idx, long long m, float* out,
                      unsigned* err, void* stream) {
    if (!src || !out || !err || rows < 0 || ld < 0 || m < 0 || (m > 0 && !idx)) return FC_ERR_ARG;
    if (rows == 0 || m == 0) return FC_OK;
    k_columns<false><<<grid_for((long long)rows * m), IO_BLOCK, 0, (cudaStream_t)stream>>>(
        const_cast<float*>(src), out, rows, ld, idx, m, err);
    return launch_status();
}

int fc_columns_scatter(float* dst, int rows, long long ld, const long long* idx, long long m, const float* cols,
                       unsigned* err, void* stream) {
    if (!dst || !cols || !err || rows < 0 || ld < 0 || m < 0 || (m > 0 && !idx)) return FC_ERR_ARG;
    if (rows == 0 || m == 0) return FC_OK;
    k_columns<true><<<grid_for((long long)rows * m), IO_BLOCK, 0, (cudaStream_t)stream>>>(
        dst, const_cast<float*>(cols), rows, ld, idx, m, err);
    return launch_status();
}

long long fc_lbm_mass_workspace_bytes(void) { return (long long)(MASS_BLOCKS + 1) * (long long)sizeof(double); }

int fc_lbm_mass(const void* pop, int storage, const uint8_t* flags, long long n_cells, void* workspace,
                long long workspace_bytes, double* result, void* stream) {
    if (!pop || !workspace || !result || n_cells < 1 || storage < ST_F32 || storage > ST_BF16S) return FC_ERR_ARG;
    if (workspace_bytes < fc_lbm_mass_workspace_bytes()) return FC_ERR_ARG;
    long long b = (n_cells + IO_BLOCK - 1) / IO_BLOCK;
    if (b > MASS_BLOCKS) b = MASS_BLOCKS;
    double* part = reinterpret_cast<double*>(workspace);
    cudaStream_t st = (cudaStream_t)stream;
    switch (storage) {
        case ST_F32: k_mass<ST_F32><<<(unsigned)b, IO_BLOCK, 0, st>>>(pop, flags, n_cells, part); break;
        case ST_F16S: k_mass<ST_F16S><<<(unsigned)b, IO_BLOCK, 0, st>>>(pop, flags, n_cells, part); break;
        default: k_mass<ST_BF16S><<<(unsigned)b, IO_BLOCK, 0, st>>>(pop, flags, n_cells, part); break;
    }
    int rc = launch_status();
    if (rc) return rc;
    k_mass_sum<<<1, IO_BLOCK, 0, st>>>(part, (int)b, result);
    return launch_status();
}

}  // extern "C"
