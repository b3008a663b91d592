// fc_common.cuh -- shared D3Q19 constants, storage codecs and status words for
// the fluxcore3d_gb300 kernels (sm_103a).
//
// Lattice layout (identical to the reference solver's population tensor
// f[19, nx, ny, nz], solver/lbm_kernels.cu:6-9): population q of cell
// flat = i*ny*nz + j*nz + k lives at q*N + flat.  Direction order, opposites
// and the 8-digit decimal weights follow solver/lbm_kernels.cu:59-71; the
// weights are kept as those literals (not 1/18, 1/36 rounded) because the
// reference kernels use them and bit parity of rest-state cells needs them.
#pragma once
#include <cuda_runtime.h>
#include <cuda_fp16.h>
#include <cuda_bf16.h>
#include <stdint.h>

namespace fc {

// ---- D3Q19 velocity set ---------------------------------------------------
// q : 0 rest | 1 +x 2 -x 3 +y 4 -y 5 +z 6 -z | 7..10 xy edges | 11..14 xz | 15..18 yz
__host__ __device__ constexpr int cx(int q) {
    return (q == 1 || q == 7 || q == 8 || q == 11 || q == 12) ? 1
         : (q == 2 || q == 9 || q == 10 || q == 13 || q == 14) ? -1 : 0;
}
__host__ __device__ constexpr int cy(int q) {
    return (q == 3 || q == 7 || q == 9 || q == 15 || q == 16) ? 1
         : (q == 4 || q == 8 || q == 10 || q == 17 || q == 18) ? -1 : 0;
}
__host__ __device__ constexpr int cz(int q) {
    return (q == 5 || q == 11 || q == 13 || q == 15 || q == 17) ? 1
         : (q == 6 || q == 12 || q == 14 || q == 16 || q == 18) ? -1 : 0;
}
__host__ __device__ constexpr int opp(int q) {
    return q == 0 ? 0 : (q <= 6 ? ((q & 1) ? q + 1 : q - 1)
                       : (q <= 10 ? 17 - q : (q <= 14 ? 25 - q : 33 - q)));
}
// Lattice weights as 8-digit decimals (see header comment).
__host__ __device__ constexpr float wq(int q) {
    return q == 0 ? 0.33333333f : (q <= 6 ? 0.05555556f : 0.02777778f);
}
// Component of c_q along axis a (0=x,1=y,2=z).
__host__ __device__ constexpr int cax(int q, int a) {
    return a == 0 ? cx(q) : (a == 1 ? cy(q) : cz(q));
}

// ---- status / error word --------------------------------------------------
// Every entry point returns an int status; kernels that detect bad input set
// bits in a device error word that the host reads when it already syncs.
enum Status : int {
    FC_OK = 0,
    FC_ERR_ARG = 1,        // bad argument (null pointer, size, mode)
    FC_ERR_LAUNCH = 2,     // cudaGetLastError after launch was not cudaSuccess
    FC_ERR_UNSUPPORTED = 3, // valid but not implemented combination
    FC_ERR_TOO_LARGE = 4    // request exceeds a fixed capacity of the library
};
enum DevErr : unsigned {
    DEV_ERR_INDEX = 1u,      // an index read from a table was out of range
    DEV_ERR_NONFINITE = 2u,  // a non-finite value was produced
    DEV_ERR_TIMEOUT = 4u,    // a bounded wait on an mbarrier gave up (staged copies never landed)
};

// ---- cell flag byte used by the fused step --------------------------------
enum CellFlag : uint8_t {
    CF_SOLID = 1,     // flow solid: populations pinned to W, never touched
    CF_LINK = 2,      // cell owns >=1 interpolated-bounce-back link
    CF_DEFER = 4,     // cell lies on an inlet/outlet plane handled after the pass
    CF_WRITE_S = 8,   // post-stream populations must be exported to f (BC input)
};

// ---- population storage codecs --------------------------------------------
// F32: plain FP32 (parity mode).  F16S / BF16S: the stored value is f - w_q
// (shifted) so that the 10/7 mantissa bits describe the deviation from rest.
enum StorageKind : int { ST_F32 = 0, ST_F16S = 1, ST_BF16S = 2 };

template <int KIND> struct Store;
template <> struct Store<ST_F32> {
    using T = float;
    static __device__ __forceinline__ float load(const T* p, int q) { (void)q; return __ldg(p); }
    static __device__ __forceinline__ void store(T* p, int q, float v) { (void)q; *p = v; }
    static constexpr int bytes = 4;
};
template <> struct Store<ST_F16S> {
    using T = __half;
    static __device__ __forceinline__ float load(const T* p, int q) {
        return __half2float(__ldg(p)) + wq(q);
    }
    static __device__ __forceinline__ void store(T* p, int q, float v) {
        *p = __float2half_rn(v - wq(q));
    }
    static constexpr int bytes = 2;
};
template <> struct Store<ST_BF16S> {
    using T = __nv_bfloat16;
    static __device__ __forceinline__ float load(const T* p, int q) {
        return __bfloat162float(__ldg(p)) + wq(q);
    }
    static __device__ __forceinline__ void store(T* p, int q, float v) {
        *p = __float2bfloat16_rn(v - wq(q));
    }
    static constexpr int bytes = 2;
};

inline int launch_status() {
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? FC_OK : FC_ERR_LAUNCH;
}

}  // namespace fc
