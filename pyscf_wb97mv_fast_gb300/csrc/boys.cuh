// FP32 Boys function F_0..F_L used by the COSX kernels (device only).
#pragma once
#include <cuda_runtime.h>

#include "f32x2.cuh"

namespace wb {

// ---------------------------------------------------------------------------
// FP32 Boys F_0 .. F_L (L <= 6).
//   T < 36: Taylor expansion about the nearest node T_k = k/4,
//     F_n(T) = sum_{j=0..6} F_{n+j}(T_k) (-h)^j / j!,  h = T - T_k exact,
//     with F_n(T_k) carried as hi + lo and the lo part added to the tail
//     before the single final addition (the switch at 36 and the node
//     spacing follow the reference, gpu/boys.py:14-44).
//   T >= 36: the asymptotic form F_n = Gamma(n + 1/2) / (2 T^(n + 1/2)),
//     evaluated on the mantissa of an exact split T = m 4^e (boys_asym).
// Row layout of the Taylor table (5 float4):
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
// V = float (one point) or float2 (a lane's two points, packed); the two
// forms give bitwise the same values.
template<int L, typename V>
__device__ __forceinline__ void far_r000_v(const V r2, const float k0h_s,
                                           const float k0l_s, V* R) {
    const V k0h = v_const<V>(k0h_s), k0l = v_const<V>(k0l_s);
    const V s0 = v_rsqrt(r2);
    const V a = v_mul(s0, s0);
    const V a_lo = v_fma(s0, s0, v_neg(a));
    // 1 - r2 s0^2 with the square exact
    const V rr = v_fma(v_neg(r2), a_lo, v_fma(v_neg(r2), a, v_const<V>(1.0f)));
    const V sh = s0, sl = v_mul(v_mul(v_const<V>(0.5f), s0), rr);
    R[0] = v_fma(k0h, sh, v_fma(k0h, sl, v_mul(k0l, sh)));
    if (L >= 1) {
        const V uh = v_mul(sh, sh);
        const V ul = v_fma(v_mul(v_const<V>(2.0f), sh), sl, v_fma(sh, sh, v_neg(uh)));
        V th = v_mul(k0h, sh);
        V tl = v_add(v_fma(k0h, sh, v_neg(th)), v_fma(k0h, sl, v_mul(k0l, sh)));
#pragma unroll
        for (int n = 1; n <= L; ++n) {
            // t *= u, then R000_n = t (-(2n-1)!!)
            const V p = v_mul(th, uh);
            const V e = v_add(v_fma(th, uh, v_neg(p)), v_fma(th, ul, v_mul(tl, uh)));
            th = v_add(p, e);
            tl = v_sub(e, v_sub(th, p));
            float dfs = 1.0f;
            for (int j = 1; j <= n; ++j) dfs *= -(float)(2 * j - 1);
            const V df = v_const<V>(dfs);
            const V q = v_mul(th, df);
            R[n] = v_add(q, v_fma(tl, df, v_fma(th, df, v_neg(q))));
        }
    }
}

template<int L>
__device__ __forceinline__ void far_r000(const float r2, const float k0h,
                                         const float k0l, float* R) {
    far_r000_v<L, float>(r2, k0h, k0l, R);
}

// Double-float helpers of the asymptotic branch: a value is hi + lo with
// |lo| <= ulp(hi)/2.  df_prod is Dekker's product with an FMA for the exact
// error of hi*hi and a renormalisation (about 44 significant bits).
struct DFloat { float hi, lo; };

__device__ __forceinline__ DFloat df_prod(const DFloat x, const DFloat y) {
    const float top = x.hi * y.hi;
    const float err = fmaf(x.hi, y.hi, -top) + fmaf(x.lo, y.hi, x.hi * y.lo);
    const float hi = top + err;
    return DFloat{hi, err - (hi - top)};
}

// T >= 36 (finite): F_n(T) = g_n T^-(n + 1/2), g_n = Gamma(n + 1/2)/2.  The
// neglected term of the exact F_n is below exp(-T)/(2T) < 4e-18 there.
//
// T is split exactly as m 4^e with m in [1, 4) by moving 2e out of the
// binary exponent.  Then F_n = [g_n r^(2n + 1)] 2^(-e (2n + 1)), r = m^-1/2
// in (1/2, 1].  The bracket is at least g_n 2^-13 and at most g_n, so its
// double-float evaluation never meets a subnormal error term whatever T is;
// it is rounded once, and the power of two is applied exactly (a result
// below the normal range rounds as any subnormal product would).
//   r: rsqrt plus one Newton step, r = r0 + r0 (1 - m r0^2) / 2, the
//      residual taken with the exact square of r0 (about 44 bits);
//   r^(2n + 1): running double-float products by r^2;
//   g_n: (2n - 1)!! sqrt(pi) / 2^(n + 1) as hi + lo (FP32 pairs of the
//      exact values, rounded from 60-digit decimals).
// Maximum error: one rounding (0.5 ulp) plus about 2^-40 relative.
template<int L>
__device__ __forceinline__ void boys_asym(const float T, float* F) {
    const int bits = __float_as_int(T);
    const int e = (((bits >> 23) & 0xff) - 127) >> 1;   // T >= 36: e >= 2
    const float m = __int_as_float(bits - (e << 24));    // T / 4^e in [1, 4)
    const float r0 = rsqrtf(m);
    const float sq = r0 * r0;
    const float resid = fmaf(-m, sq, 1.0f) - m * fmaf(r0, r0, -sq);
    const DFloat r = DFloat{r0, 0.5f * r0 * resid};
    const DFloat r2 = df_prod(r, r);
    const float step = __int_as_float((127 - 2 * e) << 23);   // 2^-2e, exact
    float scale = __int_as_float((127 - e) << 23);            // 2^-e
    constexpr float gh[7] = {8.862269521e-01f, 4.431134760e-01f, 6.646701694e-01f,
                             1.661675453e+00f, 5.815864086e+00f, 2.617138863e+01f,
                             1.439426422e+02f};
    constexpr float gl[7] = {-2.662319964e-08f, -1.331159982e-08f, 2.473608340e-08f,
                             3.203788523e-08f, 1.121326036e-07f, 2.661781195e-07f,
                             -3.304391839e-06f};
    DFloat pw = r;                                  // r^(2n + 1)
#pragma unroll
    for (int n = 0; n <= L; ++n) {
        const DFloat v = df_prod(DFloat{gh[n], gl[n]}, pw);
        F[n] = (v.hi + v.lo) * scale;
        if (n < L) {
            pw = df_prod(pw, r2);
            scale *= step;
        }
    }
}

template<int L>
__device__ __forceinline__ void boys_fp32(float T, float* F,
                                          const float4* __restrict__ tab) {
    if (!(T > 0.0f)) T = 0.0f;
    if (T < WB_BOYS_TSWITCH) {
        boys_taylor<L>(T, F, tab);
    } else if (T < INFINITY) {
        boys_asym<L>(T, F);
    } else {
#pragma unroll
        for (int n = 0; n <= L; ++n) F[n] = 0.0f;
    }
}

}  // namespace wb
