// fc_vec.cuh -- one-cell (f1) and two-cell (f2) FP32 arithmetic for the
// shifted-variable collision.
//
// f2 carries the same quantity for two neighbouring cells and maps every add,
// multiply and fused multiply-add onto the packed FP32 instructions of sm_100+
// (__fadd2_rn, __fmul2_rn, __ffma2_rn): one instruction advances both cells.
// Every operation of both types is an explicitly rounded IEEE operation -- f1
// uses __fadd_rn / __fmul_rn / __fmaf_rn, which the compiler never contracts --
// so a cell gives bit-identical results whether it is collided alone (f1) or as
// one lane of a pair (f2).  Fused multiply-adds appear only where fma() is
// written.
#pragma once
#include <cuda_runtime.h>

namespace fc {

struct f1 {
    float v;
};
struct f2 {
    float2 v;
};

__device__ __forceinline__ f1 operator+(f1 a, f1 b) { return {__fadd_rn(a.v, b.v)}; }
__device__ __forceinline__ f1 operator-(f1 a, f1 b) { return {__fsub_rn(a.v, b.v)}; }
__device__ __forceinline__ f1 operator*(f1 a, f1 b) { return {__fmul_rn(a.v, b.v)}; }
__device__ __forceinline__ f1 operator*(float s, f1 a) { return {__fmul_rn(s, a.v)}; }
__device__ __forceinline__ f1 operator+(f1 a, float s) { return {__fadd_rn(a.v, s)}; }
__device__ __forceinline__ f1 fma(f1 a, f1 b, f1 c) { return {__fmaf_rn(a.v, b.v, c.v)}; }
__device__ __forceinline__ f1 fma(float s, f1 b, f1 c) { return {__fmaf_rn(s, b.v, c.v)}; }

__device__ __forceinline__ float2 bc2(float s) { return make_float2(s, s); }
__device__ __forceinline__ f2 operator+(f2 a, f2 b) { return {__fadd2_rn(a.v, b.v)}; }
// a - b as fma(b, -1, a): b * -1 is exact, so the single rounding equals that of a - b
__device__ __forceinline__ f2 operator-(f2 a, f2 b) { return {__ffma2_rn(b.v, bc2(-1.f), a.v)}; }
__device__ __forceinline__ f2 operator*(f2 a, f2 b) { return {__fmul2_rn(a.v, b.v)}; }
__device__ __forceinline__ f2 operator*(float s, f2 a) { return {__fmul2_rn(bc2(s), a.v)}; }
__device__ __forceinline__ f2 operator+(f2 a, float s) { return {__fadd2_rn(a.v, bc2(s))}; }
__device__ __forceinline__ f2 fma(f2 a, f2 b, f2 c) { return {__ffma2_rn(a.v, b.v, c.v)}; }
__device__ __forceinline__ f2 fma(float s, f2 b, f2 c) { return {__ffma2_rn(bc2(s), b.v, c.v)}; }

template <class V> __device__ __forceinline__ V splat(float s);
template <> __device__ __forceinline__ f1 splat<f1>(float s) { return {s}; }
template <> __device__ __forceinline__ f2 splat<f2>(float s) { return {bc2(s)}; }

// per-lane operations without a packed form
__device__ __forceinline__ f1 rcp(f1 a) { return {__frcp_rn(a.v)}; }
__device__ __forceinline__ f2 rcp(f2 a) { return {make_float2(__frcp_rn(a.v.x), __frcp_rn(a.v.y))}; }
__device__ __forceinline__ f1 vsqrt(f1 a) { return {__fsqrt_rn(a.v)}; }
__device__ __forceinline__ f2 vsqrt(f2 a) { return {make_float2(__fsqrt_rn(a.v.x), __fsqrt_rn(a.v.y))}; }
__device__ __forceinline__ f1 vmax(f1 a, f1 b) { return {fmaxf(a.v, b.v)}; }
__device__ __forceinline__ f2 vmax(f2 a, f2 b) { return {make_float2(fmaxf(a.v.x, b.v.x), fmaxf(a.v.y, b.v.y))}; }
__device__ __forceinline__ f1 vmin(f1 a, float s) { return {fminf(a.v, s)}; }
__device__ __forceinline__ f2 vmin(f2 a, float s) { return {make_float2(fminf(a.v.x, s), fminf(a.v.y, s))}; }

// lane access (lane 0 of an f1 is its value)
__device__ __forceinline__ float lane(f1 a, int) { return a.v; }
__device__ __forceinline__ float lane(f2 a, int l) { return l ? a.v.y : a.v.x; }
__device__ __forceinline__ void set_lane(f1& a, int, float x) { a.v = x; }
__device__ __forceinline__ void set_lane(f2& a, int l, float x) {
    if (l) a.v.y = x;
    else a.v.x = x;
}

}  // namespace fc
