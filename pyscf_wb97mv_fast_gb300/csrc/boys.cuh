// FP32 Boys function F_0..F_L used by the COSX kernels (device only).
#pragma once
#include <cuda_runtime.h>

namespace wb {

// ---------------------------------------------------------------------------
// FP32 Boys F_0 .. F_L (L <= 6).
//   T < 36: Taylor expansion about the nearest node T_k = k/4,
//     F_n(T) = sum_{j=0..6} F_{n+j}(T_k) (-h)^j / j!,  h = T - T_k exact,
//     with F_n(T_k) carried as hi + lo and the lo part added to the tail
//     before the single final addition.
//   T >= 36: the asymptotic form F_n = (2n-1)!!/2^(n+1) sqrt(pi) T^-(n+1/2)
//     in double-float arithmetic (FMA error terms), scaled by 2^100 so that
//     no error term becomes subnormal; T > 1e30 gives 0.
// The same algorithm as the reference (gpu/boys.py:14-44, :121-168); the
// table layout and the Taylor evaluation order are this library's.
// Row layout (5 float4):
//   [h0 h1 h2 h3 | h4 h5 h6 l0 | h7 l1 h8 l2 | h9 l3 h10 l4 | h11 l5 h12 l6]
// ---------------------------------------------------------------------------
#define WB_BOYS_TSWITCH 36.0f

// The T < 36 branch alone (T in [0, 36.06)): Taylor about the nearest node,
// F_n(T) = sum_j F_{n+j}(T_k) (-h)^j / j!, in nested form:
//   t = F_{n+6};  t = F_{n+j} + t (-h) / (j + 1)  for j = 5 .. 1;
//   F_n = F_n,hi + (F_n,lo + (-h) t)
// (the (-h)/(j+1) are formed once for every order; one dependent FMA chain
// per order; the lo part joins before the single final addition).
template<int L>
__device__ __forceinline__ void boys_taylor(float T, float* F,
                                            const float4* __restrict__ tab) {
    T = fmaxf(T, 0.0f);
    const int k = __float2int_rn(T * 4.0f);
    const float mh = fmaf(0.25f, (float)k, -T);           // -h, exact
    const float m2 = mh * 0.5f, m3 = mh * (1.0f / 3.0f), m4 = mh * 0.25f;
    const float m5 = mh * 0.2f, m6 = mh * (1.0f / 6.0f);
    const float4* row = tab + k * 5;
    float hv[13], lv[7];
    {
        const float4 a = row[0], b = row[1];
        hv[0] = a.x; hv[1] = a.y; hv[2] = a.z; hv[3] = a.w;
        hv[4] = b.x; hv[5] = b.y; hv[6] = b.z; lv[0] = b.w;
    }
    if (L >= 1) {
        const float4 c = row[2];
        hv[7] = c.x; lv[1] = c.y; hv[8] = c.z; lv[2] = c.w;
    }
    if (L >= 3) {
        const float4 d = row[3];
        hv[9] = d.x; lv[3] = d.y; hv[10] = d.z; lv[4] = d.w;
    }
    if (L >= 5) {
        const float4 e = row[4];
        hv[11] = e.x; lv[5] = e.y; hv[12] = e.z; lv[6] = e.w;
    }
#pragma unroll
    for (int n = 0; n <= L; ++n) {
        float t = fmaf(hv[n + 6], m6, hv[n + 5]);
        t = fmaf(t, m5, hv[n + 4]);
        t = fmaf(t, m4, hv[n + 3]);
        t = fmaf(t, m3, hv[n + 2]);
        t = fmaf(t, m2, hv[n + 1]);
        F[n] = hv[n] + fmaf(mh, t, lv[n]);
    }
}

// Far field, T >= 36 (erf(sqrt T) = 1 to FP64 precision): the Hermite
// sources R000_n = c_n F_n(T) are (-1)^n (2n-1)!! K0 r^-(2n+1), K0 = c_0
// sqrt(pi) / (2 sqrt(theta p)) per primitive pair (hi + lo).  1/r is carried
// in double-float (rsqrt and one Newton correction), the powers and the
// odd double factorials in double-float, one rounding per R000_n -- the
// same accuracy as c_n times the asymptotic F_n in double-float.
template<int L>
__device__ __forceinline__ void far_r000(const float r2, const float k0h,
                                         const float k0l, float* R) {
    const float s0 = rsqrtf(r2);
    const float a = s0 * s0;
    const float a_lo = fmaf(s0, s0, -a);
    const float rr = fmaf(-r2, a, 1.0f) - r2 * a_lo;
    const float sh = s0, sl = 0.5f * s0 * rr;
    R[0] = fmaf(k0h, sh, fmaf(k0h, sl, k0l * sh));
    if (L >= 1) {
        const float uh = sh * sh;
        const float ul = fmaf(sh, sh, -uh) + 2.0f * sh * sl;
        float th = k0h * sh;
        float tl = fmaf(k0h, sh, -th) + fmaf(k0h, sl, k0l * sh);
#pragma unroll
        for (int n = 1; n <= L; ++n) {
            // t *= u, then R000_n = t (-(2n-1)!!)
            const float p = th * uh;
            const float e = fmaf(th, uh, -p) + fmaf(th, ul, tl * uh);
            th = p + e;
            tl = e - (th - p);
            float df = 1.0f;
            for (int j = 1; j <= n; ++j) df *= -(float)(2 * j - 1);
            const float q = th * df;
            R[n] = q + (fmaf(th, df, -q) + tl * df);
        }
    }
}

template<int L>
__device__ __forceinline__ void boys_fp32(float T, float* F,
                                          const float4* __restrict__ tab) {
    if (!(T > 0.0f)) T = 0.0f;
    if (T < WB_BOYS_TSWITCH) {
        boys_taylor<L>(T, F, tab);
    } else if (T > 1e30f) {
#pragma unroll
        for (int n = 0; n <= L; ++n) F[n] = 0.0f;
    } else {
        // s = 1/sqrt(T) as s_hi + s_lo: rsqrtf and one Newton correction
        const float s0 = rsqrtf(T);
        const float a = s0 * s0;
        const float a_lo = fmaf(s0, s0, -a);
        const float r = fmaf(-T, a, 1.0f) - T * a_lo;
        const float s_hi = s0, s_lo = 0.5f * s0 * r;
        const float u_hi = s_hi * s_hi;
        const float u_lo = fmaf(s_hi, s_hi, -u_hi) + 2.0f * s_hi * s_lo;
        // sqrt(pi)/2 = 0.886226925452758... as hi + lo, scaled by 2^100
        const float c_hi = 0.886226952075958252f * 1.2676506002282294e30f;
        const float c_lo = -2.662319964e-08f * 1.2676506002282294e30f;
        float f_hi = c_hi * s_hi;
        float f_lo = fmaf(c_hi, s_hi, -f_hi) + (c_hi * s_lo + c_lo * s_hi);
        F[0] = (f_hi + f_lo) * 7.888609052210118e-31f;
#pragma unroll
        for (int n = 1; n <= L; ++n) {
            const float cc = (float)n - 0.5f;
            const float cu_hi = cc * u_hi;
            const float cu_lo = fmaf(cc, u_hi, -cu_hi) + cc * u_lo;
            const float p = f_hi * cu_hi;
            const float e = fmaf(f_hi, cu_hi, -p) + (f_hi * cu_lo + f_lo * cu_hi);
            f_hi = p + e;
            f_lo = e - (f_hi - p);
            F[n] = f_hi * 7.888609052210118e-31f;
        }
    }
}

}  // namespace wb
