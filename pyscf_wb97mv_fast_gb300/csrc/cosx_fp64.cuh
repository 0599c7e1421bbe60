// Plain FP64 form of the fused screen + G kernels (templates shared by
// cosx_fp64.cu and cosx_fp64_f.cu): the same task set (the
// reference's locked bound on 32-point blocks, tol / 1.001) and the same
// McMurchie-Davidson algorithm as the FP32 class kernels, with every
// arithmetic step in FP64 and G accumulated in FP64.  It is the comparison
// point of the mixed-precision path and the operator of an FP64 tail; the
// reference runs that tail through stock PySCF on the CPU
// (staging/schedule.py:329-334).
//
// One warp owns one 32-point block (one point per lane) and walks its
// class's shell pairs in order; 32 pairs at a time each lane evaluates one
// pair's bound and a ballot keeps the warp on the kept ones.  Per task and
// point: F_A, F_B -> Cartesian (c2s^T F), per primitive pair the Boys
// values (FP64 Taylor table + downward recursion, or the asymptotic form
// with upward recursion), R_tuv in place, the Hermite sums, and the
// F-first accumulation ya += A fb, yb += A^T fa; the task ends with
// G_A += c2s ya and G_B += c2s yb (diagonal pairs: G_A += (c2s ya + c2s
// yb) / 2, the symmetrised block).  Each lane owns its point's column of G
// and the classes run one after another on one stream, so every element of
// G has one writer and a fixed summation order.
#pragma once
#include <algorithm>
#include <cuda_runtime.h>

#include "cosx_kernels.cuh"
#include "cosx_fp64.hpp"

namespace wb {
namespace f64 {

constexpr int kF64Threads = 128;
constexpr int kTaylor = 12;              // terms of the Boys Taylor series

constexpr __host__ __device__ int ncart_c(int l) { return (l + 1) * (l + 2) / 2; }
constexpr __host__ __device__ int nr_c(int L) { return (L + 1) * (L + 2) * (L + 3) / 6; }
// packed index of R_tuv (t + u + v <= L): v-major, then u, then t
constexpr __host__ __device__ int ridx(int L, int t, int u, int v) {
    int k = 0;
    for (int vv = 0; vv < v; ++vv)
        for (int uu = 0; uu <= L - vv; ++uu) k += L - vv - uu + 1;
    for (int uu = 0; uu < u; ++uu) k += L - v - uu + 1;
    return k + t;
}
// Cartesian exponents of component c of shell l (libcint order)
constexpr __host__ __device__ int cx(int l, int c) {
    int n = 0;
    for (int x = l; x >= 0; --x)
        for (int y = l - x; y >= 0; --y) {
            if (n == c) return x;
            ++n;
        }
    return 0;
}
constexpr __host__ __device__ int cy(int l, int c) {
    int n = 0;
    for (int x = l; x >= 0; --x)
        for (int y = l - x; y >= 0; --y) {
            if (n == c) return y;
            ++n;
        }
    return 0;
}
constexpr __host__ __device__ int cz(int l, int c) { return l - cx(l, c) - cy(l, c); }
// offset of E^{i,j}_0 inside one axis block ([i][j][t], j <= lb)
constexpr __host__ __device__ int eoff(int lb, int i, int j) {
    int k = 0;
    for (int ii = 0; ii < i; ++ii)
        for (int jj = 0; jj <= lb; ++jj) k += ii + jj + 1;
    for (int jj = 0; jj < j; ++jj) k += i + jj + 1;
    return k;
}
constexpr __host__ __device__ int eaxis(int la, int lb) {
    return eoff(lb, la + 1, 0);
}

// c2s^T v (Cartesian components of a spherical vector) and c2s y
template<int L>
__device__ __forceinline__ void to_cart(const double* __restrict__ c2s,
                                        const double* s, double* c) {
    if constexpr (L <= 1) {
#pragma unroll
        for (int i = 0; i < ncart_c(L); ++i) c[i] = s[i];
    } else {
#pragma unroll
        for (int i = 0; i < ncart_c(L); ++i) {
            double a = 0.0;
#pragma unroll
            for (int m = 0; m < 2 * L + 1; ++m)
                a = fma(c2s[(L - 2) * 30 + i * (2 * L + 1) + m], s[m], a);
            c[i] = a;
        }
    }
}
template<int L>
__device__ __forceinline__ double to_sph(const double* __restrict__ c2s,
                                        const double* y, const int m) {
    if constexpr (L <= 1) {
        return y[m];
    } else {
        double a = 0.0;
#pragma unroll
        for (int i = 0; i < ncart_c(L); ++i)
            a = fma(c2s[(L - 2) * 30 + i * (2 * L + 1) + m], y[i], a);
        return a;
    }
}

// F_0 .. F_L at T in FP64.  T < 36: Taylor series of F_L about the nearest
// node k/4 (|dT| <= 1/8, kTaylor terms: truncation below 1e-20 relative)
// from the table tab[k][m] = F_m(k/4), then the downward recursion
// F_n = (2T F_{n+1} + e^-T) / (2n + 1).  T >= 36: erf(sqrt T) = 1 in FP64,
// F_0 = sqrt(pi / T) / 2 and the upward recursion F_{n+1} = ((2n+1) F_n -
// e^-T) / (2T), stable for T > n.
template<int L>
__device__ __forceinline__ void boys64(const double T, const double* __restrict__ tab,
                                       double* F) {
    if (T < 36.0) {
        const int k = __double2int_rn(T * 4.0);
        const double x = 0.25 * k - T;
        const double* row = tab + k * kBoys64Cols + L;
        double s = row[kTaylor - 1];
#pragma unroll
        for (int j = kTaylor - 1; j >= 1; --j) s = fma(s * x, 1.0 / j, row[j - 1]);
        F[L] = s;
        if constexpr (L > 0) {
            const double e = exp(-T);
#pragma unroll
            for (int n = L - 1; n >= 0; --n) F[n] = fma(2.0 * T, F[n + 1], e) * (1.0 / (2 * n + 1));
        }
    } else {
        F[0] = 0.88622692545275801365 * rsqrt(T);
        if constexpr (L > 0) {
            const double e = exp(-T);
            const double h = 0.5 / T;
#pragma unroll
            for (int n = 0; n < L; ++n) F[n + 1] = ((2 * n + 1) * F[n] - e) * h;
        }
    }
}

// R_tuv (t + u + v <= L) at PC = (x, y, z) from r0[n] = R_000^(n), levels
// L .. 0 in place (each level reads only the level above)
template<int L>
__device__ __forceinline__ void fill_r64(const double* r0, const double x,
                                         const double y, const double z, double* R) {
#pragma unroll
    for (int i = 0; i < nr_c(L); ++i) R[i] = 0.0;
#pragma unroll
    for (int n = L; n >= 0; --n) {
        const int m = L - n;
#pragma unroll
        for (int u = 0; u <= L; ++u)
#pragma unroll
            for (int v = 0; v <= L; ++v)
#pragma unroll
                for (int t = L; t >= 1; --t)
                    if (u < m && v < m - u && t <= m - u - v)
                        R[ridx(L, t, u, v)] =
                            (t == 1 ? 0.0 : (t - 1) * R[ridx(L, t >= 2 ? t - 2 : 0, u, v)]) +
                            x * R[ridx(L, t - 1, u, v)];
#pragma unroll
        for (int v = 0; v <= L; ++v)
#pragma unroll
            for (int u = L; u >= 1; --u)
                if (v < m && u <= m - v)
                    R[ridx(L, 0, u, v)] =
                        (u == 1 ? 0.0 : (u - 1) * R[ridx(L, 0, u >= 2 ? u - 2 : 0, v)]) +
                        y * R[ridx(L, 0, u - 1, v)];
#pragma unroll
        for (int v = L; v >= 1; --v)
            if (v <= m)
                R[ridx(L, 0, 0, v)] =
                    (v == 1 ? 0.0 : (v - 1) * R[ridx(L, 0, 0, v >= 2 ? v - 2 : 0)]) +
                    z * R[ridx(L, 0, 0, v - 1)];
        R[0] = r0[n];
    }
}

template<int LA, int LB>
__global__ void __launch_bounds__(kF64Threads)
cosx_fp64_kernel(const CosxF64Args A, const int cls, const int pair_begin,
                 const int pair_end) {
    constexpr int L = LA + LB;
    constexpr int NCA = ncart_c(LA), NCB = ncart_c(LB);
    constexpr int NA = 2 * LA + 1, NB = 2 * LB + 1;
    constexpr int NAX = eaxis(LA, LB);
    __shared__ double stab[kBoys64Nodes * kBoys64Cols];
    for (int i = threadIdx.x; i < kBoys64Nodes * kBoys64Cols; i += blockDim.x)
        stab[i] = A.boys[i];
    __syncthreads();
    const int lane = threadIdx.x & 31;
    const long long ld = A.ld;
    const int pp_begin = A.pp_begin[cls];
    const float4* __restrict__ bnd = A.bnd + pp_begin;
    const float* __restrict__ bpref = A.bpref + pp_begin;
    const double* __restrict__ Ecls = A.E + A.e_base[cls];
    const double om2 = A.omega * A.omega;
    unsigned long long kept = 0, flops = 0, ints = 0;
    for (;;) {
        int blk = 0;
        if (lane == 0) blk = atomicAdd(A.work + cls, 1);
        blk = __shfl_sync(0xffffffffu, blk, 0);
        if (blk >= A.nblk) break;
        const int g0 = blk * 32 + lane;
        const bool ok = g0 < A.npts;
        const int g = ok ? g0 : A.npts - 1;
        const double gx = A.coords[3LL * g], gy = A.coords[3LL * g + 1],
                     gz = A.coords[3LL * g + 2];
        const double* __restrict__ Fp = A.F + g;
        double* __restrict__ Gp = A.G + g;
        const float4 cr = A.blk_cr[blk];
        const float* __restrict__ ms = A.blk_msh + (long long)blk * A.nvshell;
        const int rem = A.npts - blk * 32;
        const int nvalid = rem < 32 ? rem : 32;
        for (int c0 = pair_begin; c0 < pair_end; c0 += 32) {
            const int k = c0 + lane;
            bool keep = k < pair_end;
            if (keep && A.tol > 0.0f) {
                const int2 sh = A.pshell[k];
                keep = screen_pair(A.tol, bnd, bpref, cr, A.khdr[k], A.ptau[k],
                                   fmaxf(ms[sh.x], ms[sh.y]));
            }
            unsigned mask = __ballot_sync(0xffffffffu, keep);
            if (keep) {
                flops += (unsigned long long)A.pflops[k] * nvalid;
                ints += (unsigned long long)A.pnint[k] * nvalid;
            }
            while (mask) {
                const int kk = c0 + __ffs(mask) - 1;
                mask &= mask - 1;
                ++kept;
                const int4 hdr = A.khdr[kk];
                const int ia0 = hdr.x & 0xffff, ib0 = hdr.y & 0xffff;
                const int pp0 = pp_begin + hdr.z, npp = hdr.w & 0xffff;
                const bool diag = (hdr.w >> 16) != 0;
                double sa[NA], sb[NB], fa[NCA], fb[NCB], ya[NCA], yb[NCB];
#pragma unroll
                for (int m = 0; m < NA; ++m) sa[m] = Fp[(long long)(ia0 + m) * ld];
#pragma unroll
                for (int m = 0; m < NB; ++m) sb[m] = Fp[(long long)(ib0 + m) * ld];
                to_cart<LA>(A.c2s, sa, fa);
                to_cart<LB>(A.c2s, sb, fb);
#pragma unroll
                for (int i = 0; i < NCA; ++i) ya[i] = 0.0;
#pragma unroll
                for (int i = 0; i < NCB; ++i) yb[i] = 0.0;
                for (int q = pp0; q < pp0 + npp; ++q) {
                    const double p = A.p[q], pref = A.pref[q];
                    const double X = A.P[3LL * q] - gx, Y = A.P[3LL * q + 1] - gy,
                                 Z = A.P[3LL * q + 2] - gz;
                    double th = 1.0, sth = 1.0;
                    if (A.omega > 0.0) {
                        th = om2 / (om2 + p);
                        sth = sqrt(th);
                    }
                    const double pth = p * th;
                    const double T = pth * (X * X + Y * Y + Z * Z);
                    double Fb[L + 1], r0[L + 1];
                    boys64<L>(T, stab, Fb);
                    double c = pref * sth;
#pragma unroll
                    for (int n = 0; n <= L; ++n) {
                        r0[n] = c * Fb[n];
                        c *= -2.0 * pth;
                    }
                    double R[nr_c(L)];
                    fill_r64<L>(r0, X, Y, Z, R);
                    const double* __restrict__ E = Ecls + (long long)(q - pp_begin) * 3 * NAX;
                    // the f classes keep these two loops rolled (compile time)
#pragma unroll(L <= 4 ? NCA : 1)
                    for (int a = 0; a < NCA; ++a)
#pragma unroll(L <= 4 ? NCB : 1)
                        for (int b = 0; b < NCB; ++b) {
                            const int i = cx(LA, a), j = cy(LA, a), kz = cz(LA, a);
                            const int ip = cx(LB, b), jp = cy(LB, b), kp = cz(LB, b);
                            const double* Ex = E + eoff(LB, i, ip);
                            const double* Ey = E + NAX + eoff(LB, j, jp);
                            const double* Ez = E + 2 * NAX + eoff(LB, kz, kp);
                            double s = 0.0;
#pragma unroll
                            for (int v = 0; v <= L; ++v) {
                                if (v > kz + kp) break;
                                double su = 0.0;
#pragma unroll
                                for (int u = 0; u <= L; ++u) {
                                    if (u > j + jp) break;
                                    double st = 0.0;
#pragma unroll
                                    for (int t = 0; t <= L; ++t) {
                                        if (t > i + ip) break;
                                        st = fma(Ex[t], R[ridx(L, t, u, v)], st);
                                    }
                                    su = fma(Ey[u], st, su);
                                }
                                s = fma(Ez[v], su, s);
                            }
                            ya[a] = fma(s, fb[b], ya[a]);
                            yb[b] = fma(s, fa[a], yb[b]);
                        }
                }
                if (ok) {
                    if (diag) {
                        if constexpr (LA == LB) {
#pragma unroll
                            for (int m = 0; m < NA; ++m) {
                                double* gp = Gp + (long long)(ia0 + m) * ld;
                                *gp += 0.5 * (to_sph<LA>(A.c2s, ya, m) + to_sph<LB>(A.c2s, yb, m));
                            }
                        }
                    } else {
#pragma unroll
                        for (int m = 0; m < NA; ++m) {
                            double* gp = Gp + (long long)(ia0 + m) * ld;
                            *gp += to_sph<LA>(A.c2s, ya, m);
                        }
#pragma unroll
                        for (int m = 0; m < NB; ++m) {
                            double* gp = Gp + (long long)(ib0 + m) * ld;
                            *gp += to_sph<LB>(A.c2s, yb, m);
                        }
                    }
                }
            }
        }
    }
    for (int o = 16; o > 0; o >>= 1) {
        flops += __shfl_xor_sync(0xffffffffu, flops, o);
        ints += __shfl_xor_sync(0xffffffffu, ints, o);
    }
    if (lane == 0 && kept) {
        atomicAdd(A.counters + 3 * cls + 0, kept);
        atomicAdd(A.counters + 3 * cls + 1, flops);
        atomicAdd(A.counters + 3 * cls + 2, ints);
    }
}

template<int LA, int LB>
cudaError_t run64(const CosxF64Args& a, int cls, int pb, int pe, int nsm,
                  cudaStream_t s) {
    auto k = cosx_fp64_kernel<LA, LB>;
    int occ = 0;
    cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k, kF64Threads, 0);
    if (e != cudaSuccess) return e;
    const int warps = kF64Threads / 32;
    int grid = std::max(1, nsm * std::max(occ, 1));
    grid = std::min(grid, (a.nblk + warps - 1) / warps);
    k<<<std::max(grid, 1), kF64Threads, 0, s>>>(a, cls, pb, pe);
    return cudaGetLastError();
}

}  // namespace f64
}  // namespace wb
