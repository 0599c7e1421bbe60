// Digit arithmetic of the Ozaki split (ozaki.cu, ozaki_tc.cu): the
// fixed-point conversion of FP64 values to balanced base-2^B digits, and
// the exact int64 combination of FP32 level sums back to FP32 / FP64.
#pragma once
#include <cuda_runtime.h>

#include <cstdint>

#include "ozaki.hpp"

namespace wb {

// Fixed-point digits.  A value x with |x| < 2^e becomes the integer
// q = rint(x 2^(W - 1 - e)), W = B S bits, |q| < 2^(W-1), written as
// balanced base-2^B digits q = sum_i d_i 2^(B (S-1-i)), |d_i| <= 2^(B-1),
// extracted from the least significant end with integer arithmetic only
// (the one FP64 multiply by an exact power of two and one FP64 -> int64
// conversion per element are the only FP64 operations).
constexpr int kB = kOzBits;
constexpr int kW = kOzBits * kOzSlices;

__device__ __forceinline__ double pow2(int k) {
    // exact 2^k for -1022 <= k <= 1023
    return __longlong_as_double((long long)(1023 + k) << 52);
}

__device__ __forceinline__ int exp_of_bits(unsigned long long absbits) {
    // smallest e with |x| < 2^e from the bit pattern of |x|, clamped to
    // [-400, 500]: rows whose largest entry is below 2^-400 are zero at this
    // precision, and the clamp keeps every scale factor 2^k of the kernels
    // (|k| <= 2 * 500 + 84) inside the normal FP64 range of pow2()
    const int ebits = (int)(absbits >> 52);
    int e = ebits - 1022;                           // |x| < 2^(ebits-1023+1)
    if (absbits == 0ull || e < -400) e = -400;
    return e > 500 ? 500 : e;
}

// q = rint(x 2^(W-1-e)) from the bit pattern of x with integer arithmetic:
// |x| = m 2^p (m the 53-bit significand), shifted right with round half to
// even -- the same integer as an exact FP64 scaling followed by
// round-to-nearest, without the FP64 pipe (1/64 of the FP32 rate on GB300)
__device__ __forceinline__ long long fixed_q(double x, int e) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(x);
    const int E = (int)((b >> 52) & 0x7ff);
    unsigned long long m = b & 0xfffffffffffffull;
    int p = -1074;
    if (E) { m |= 1ull << 52; p = E - 1075; }
    const int sh = p + kW - 1 - e;
    unsigned long long q = 0;
    if (m) {
        if (sh >= 0) {
            // only small m (|x| < 2^e keeps q below 2^(W-1))
            q = m << (sh < 11 ? sh : 11);
        } else if (sh > -64) {
            const int r = -sh;
            q = m >> r;
            const unsigned long long rem = m & ((1ull << r) - 1);
            const unsigned long long half = 1ull << (r - 1);
            if (rem > half || (rem == half && (q & 1ull))) ++q;
        }
    }
    return (b >> 63) ? -(long long)q : (long long)q;
}

template<int S>
__device__ __forceinline__ void digits(double x, int e, float* d) {
    // q (|q| < 2^(W-1) = 2^41) split as q = hi 2^24 + lo, lo in [0, 2^24):
    // the four low digits come from lo, the carry goes into hi, the rest
    // from hi -- 32-bit integer arithmetic throughout
    static_assert(S == 7 && kB == 6, "digit split assumes 7 x 6 bits");
    const long long q = fixed_q(x, e);
    int lo = (int)(q & 0xFFFFFF);
    int hi = (int)(q >> 24);
#pragma unroll
    for (int i = S - 1; i >= S - 4; --i) {
        const int di = ((lo + 32) & 63) - 32;
        d[i] = (float)di;
        lo = (lo - di) >> 6;
    }
    hi += lo;
#pragma unroll
    for (int i = S - 5; i >= 1; --i) {
        const int di = ((hi + 32) & 63) - 32;
        d[i] = (float)di;
        hi = (hi - di) >> 6;
    }
    d[0] = (float)hi;
}

// RN(v 2^sc) as FP32 from the int64 v with integer arithmetic (one
// rounding); results outside the normal FP32 range take the FP64 path
__device__ __forceinline__ float scaled_ll_to_float(long long v, int sc) {
    if (v == 0) return 0.0f;
    const unsigned long long a = v < 0 ? 0ull - (unsigned long long)v
                                       : (unsigned long long)v;
    const int nb = 64 - __clzll((long long)a);
    unsigned long long q;
    int e2;
    if (nb > 24) {
        int r = nb - 24;
        q = a >> r;
        const unsigned long long rem = a & ((1ull << r) - 1);
        const unsigned long long half = 1ull << (r - 1);
        if (rem > half || (rem == half && (q & 1ull))) ++q;
        if (q == (1ull << 24)) { q >>= 1; ++r; }
        e2 = r;
    } else {
        q = a << (24 - nb);
        e2 = nb - 24;
    }
    const int E = e2 + sc + 23 + 127;
    if (E <= 0 || E >= 255)
        return __double2float_rn((double)v * pow2(sc < -1000 ? -1000 : (sc > 1000 ? 1000 : sc)));
    const unsigned bits = ((unsigned)E << 23) | ((unsigned)q & 0x7fffffu) |
                          (v < 0 ? 0x80000000u : 0u);
    return __uint_as_float(bits);
}

// v 2^sc as FP64: one rounding of v to 53 bits, then an exact scaling (sc
// stays inside pow2's range for the clamped exponents of the split)
__device__ __forceinline__ double scaled_ll_to_double(long long v, int sc) {
    return (double)v * pow2(sc);
}

// the combined value in the output type of an F product (FP32 or FP64)
template<typename T> __device__ __forceinline__ T scaled_ll_to(long long v, int sc);
template<> __device__ __forceinline__ float scaled_ll_to<float>(long long v, int sc) {
    return scaled_ll_to_float(v, sc);
}
template<> __device__ __forceinline__ double scaled_ll_to<double>(long long v, int sc) {
    return scaled_ll_to_double(v, sc);
}

// value of the combined levels: sum_l C_l 2^(B (S-1-l)) as an exact int64
// (every level is an integer below 2^24 in magnitude: 32-bit conversion)
template<int S>
__device__ __forceinline__ long long combine_levels(const float* c) {
    long long acc = 0;
#pragma unroll
    for (int l = 0; l < S; ++l)
        acc += ((long long)__float2int_rn(c[l])) << (kB * (S - 1 - l));
    return acc;
}

}  // namespace wb
