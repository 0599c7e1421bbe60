// Scalar and packed (two FP32 values in one register pair, the .f32x2
// instructions of sm_100+) forms of the same FP32 operations.  The scalar
// forms are the _rn intrinsics, which the compiler never fuses into an
// FMA, and the packed ones round each half exactly as the scalar
// instruction does (x - y is x + (-y) exactly), so code written once over
// V = float or V = float2 gives bitwise the same values in both forms.
#pragma once
#include <cuda_runtime.h>

namespace wb {

__device__ __forceinline__ float2 bc2(const float a) { return make_float2(a, a); }
__device__ __forceinline__ float2 neg2(const float2 a) { return make_float2(-a.x, -a.y); }
__device__ __forceinline__ float2 add2(const float2 a, const float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 sub2(const float2 a, const float2 b) {
    return __fadd2_rn(a, neg2(b));
}
__device__ __forceinline__ float2 mul2(const float2 a, const float2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ float2 fma2(const float2 a, const float2 b, const float2 c) {
    return __ffma2_rn(a, b, c);
}

__device__ __forceinline__ float v_add(const float a, const float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float v_sub(const float a, const float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ float v_mul(const float a, const float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float v_fma(const float a, const float b, const float c) {
    return __fmaf_rn(a, b, c);
}
__device__ __forceinline__ float v_neg(const float a) { return -a; }
__device__ __forceinline__ float v_rsqrt(const float a) { return rsqrtf(a); }

__device__ __forceinline__ float2 v_add(const float2 a, const float2 b) { return add2(a, b); }
__device__ __forceinline__ float2 v_sub(const float2 a, const float2 b) { return sub2(a, b); }
__device__ __forceinline__ float2 v_mul(const float2 a, const float2 b) { return mul2(a, b); }
__device__ __forceinline__ float2 v_fma(const float2 a, const float2 b, const float2 c) {
    return fma2(a, b, c);
}
__device__ __forceinline__ float2 v_neg(const float2 a) { return neg2(a); }
__device__ __forceinline__ float2 v_rsqrt(const float2 a) {
    return make_float2(rsqrtf(a.x), rsqrtf(a.y));
}

// a warp-uniform constant in either form
template<typename V> __device__ __forceinline__ V v_const(float c);
template<> __device__ __forceinline__ float v_const<float>(const float c) { return c; }
template<> __device__ __forceinline__ float2 v_const<float2>(const float c) { return bc2(c); }

}  // namespace wb
