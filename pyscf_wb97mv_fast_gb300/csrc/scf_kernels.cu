// Device kernels of the SCF driver (wb_scf_int1e, wb_hartree):
//
//   * one-electron integrals S, T, V in FP64 (McMurchie-Davidson: Hermite
//     expansion coefficients E^{ij}_t, the kinetic operator through the
//     1-D overlaps with j +- 2, the nuclear attraction through the Hermite
//     Coulomb integrals R_tuv at each nucleus);
//   * the Hartree potential at grid points, v_H(g) = sum_{mu nu} D_{mu nu}
//     (mu nu | 1/|r - g|), in FP64 or FP32, from a per-iteration Hermite
//     density of every primitive pair.
//
// The functions are the same contracted spherical AOs as the AO evaluation
// and the COSX kernels (libcint Cartesian order, real solid harmonics,
// per-primitive normalisation in the coefficients).  The reference takes
// these pieces from PySCF (int1e_ovlp / int1e_kin / int1e_nuc and the SGX
// Coulomb build); it has no GPU counterpart.
#include <cmath>

#include "boys.cuh"
#include "cosx_fp64.cuh"
#include "generated/hartree_r.cuh"
#include "scf.hpp"

namespace wb {
namespace scf {

using f64::boys64;
using f64::cx;
using f64::cy;
using f64::cz;
using f64::ncart_c;
using f64::nr_c;
using f64::ridx;

// (ncart, nsph) row-major c2s of l = 0..3 at offsets 0, 1, 10, 40 (the
// AO evaluation's tables: the s and p angular factors included)
__constant__ double c_c2s_all[110];

__device__ __forceinline__ const double* c2s_of(int l) {
    return c_c2s_all + (l == 0 ? 0 : l == 1 ? 1 : l == 2 ? 10 : 40);
}

// 1-D Hermite expansion coefficients of x_A^i x_B^j, E[(i * kEJ + j) * kET +
// t] for i <= ni, j <= nj (t <= i + j), from E^{00}_0 = 1 by
// E^{i+1,j}_t = E^{ij}_{t-1} / (2p) + X_PA E^{ij}_t + (t + 1) E^{ij}_{t+1}
// and the same in j with X_PB (Helgaker, Jorgensen, Olsen, eq. 9.5.6).
// Run-time sizes: these kernels run once per geometry or once per SCF
// iteration, so compact code beats unrolled code.
constexpr int kEJ = 6, kET = 10;            // j <= 5, t <= 9
__device__ void hermite1d_rt(const int ni, const int nj, const double inv2p,
                             const double xpa, const double xpb, double* E) {
#pragma unroll 1
    for (int q = 0; q < (ni + 1) * kEJ * kET; ++q) E[q] = 0.0;
    E[0] = 1.0;
#pragma unroll 1
    for (int i = 1; i <= ni; ++i)
#pragma unroll 1
        for (int t = 0; t <= i; ++t) {
            const double* pr = E + (i - 1) * kEJ * kET;
            double v = xpa * pr[t];
            if (t > 0) v += inv2p * pr[t - 1];
            if (t + 1 <= i - 1) v += (t + 1) * pr[t + 1];
            E[i * kEJ * kET + t] = v;
        }
#pragma unroll 1
    for (int j = 1; j <= nj; ++j)
#pragma unroll 1
        for (int i = 0; i <= ni; ++i)
#pragma unroll 1
            for (int t = 0; t <= i + j; ++t) {
                const double* pr = E + (i * kEJ + j - 1) * kET;
                double v = xpb * pr[t];
                if (t > 0) v += inv2p * pr[t - 1];
                if (t + 1 <= i + j - 1) v += (t + 1) * pr[t + 1];
                E[(i * kEJ + j) * kET + t] = v;
            }
}

// Cartesian exponents of component c of shell l (libcint order)
__device__ __forceinline__ void cart_xyz(const int l, const int c, int& x, int& y,
                                         int& z) {
    int n = 0;
#pragma unroll 1
    for (int a = l; a >= 0; --a)
#pragma unroll 1
        for (int b = l - a; b >= 0; --b) {
            if (n == c) { x = a; y = b; z = l - a - b; return; }
            ++n;
        }
    x = y = z = 0;
}

// R_tuv (t + u + v <= L) at PC from r0[n] = R_000^(n), run-time L, packed
// like ridx: levels L .. 0 in place (each level reads only the one above)
__device__ void fill_r_rt(const int L, const double* r0, const double x,
                          const double y, const double z, double* R);

// packed R index with run-time arguments (the one-electron kernel's sums)
__device__ __forceinline__ int ridx_rt(int L, int t, int u, int v) {
    int k = 0;
    for (int vv = 0; vv < v; ++vv) k += (L - vv + 1) * (L - vv + 2) / 2;
    for (int uu = 0; uu < u; ++uu) k += L - v - uu + 1;
    return k + t;
}

// -- one-electron integrals ----------------------------------------------------

// packed R index with run-time arguments
__device__ void fill_r_rt(const int L, const double* r0, const double x,
                          const double y, const double z, double* R) {
#pragma unroll 1
    for (int i = 0; i < (L + 1) * (L + 2) * (L + 3) / 6; ++i) R[i] = 0.0;
#pragma unroll 1
    for (int n = L; n >= 0; --n) {
        const int m = L - n;
#pragma unroll 1
        for (int v = 0; v < m; ++v)
#pragma unroll 1
            for (int u = 0; u < m - v; ++u)
#pragma unroll 1
                for (int t = m - u - v; t >= 1; --t)
                    R[ridx_rt(L, t, u, v)] =
                        (t >= 2 ? (t - 1) * R[ridx_rt(L, t - 2, u, v)] : 0.0) +
                        x * R[ridx_rt(L, t - 1, u, v)];
#pragma unroll 1
        for (int v = 0; v < m; ++v)
#pragma unroll 1
            for (int u = m - v; u >= 1; --u)
                R[ridx_rt(L, 0, u, v)] =
                    (u >= 2 ? (u - 1) * R[ridx_rt(L, 0, u - 2, v)] : 0.0) +
                    y * R[ridx_rt(L, 0, u - 1, v)];
#pragma unroll 1
        for (int v = m; v >= 1; --v)
            R[ridx_rt(L, 0, 0, v)] =
                (v >= 2 ? (v - 1) * R[ridx_rt(L, 0, 0, v - 2)] : 0.0) +
                z * R[ridx_rt(L, 0, 0, v - 1)];
        R[0] = r0[n];
    }
}

// FP64 Boys F_0..F_L at T with run-time L (the FP64 table form of boys64)
__device__ void boys_rt(const int L, const double T, const double* tab, double* F) {
    if (T < 36.0) {
        const int k = __double2int_rn(T * 4.0);
        const double x = 0.25 * k - T;
        const double* row = tab + k * kBoys64Cols + L;
        double s = row[f64::kTaylor - 1];
#pragma unroll 1
        for (int j = f64::kTaylor - 1; j >= 1; --j) s = fma(s * x, 1.0 / j, row[j - 1]);
        F[L] = s;
        const double e = exp(-T);
#pragma unroll 1
        for (int n = L - 1; n >= 0; --n) F[n] = fma(2.0 * T, F[n + 1], e) / (2 * n + 1);
    } else {
        F[0] = 0.88622692545275801365 * rsqrt(T);
        const double e = exp(-T);
        const double h = 0.5 / T;
#pragma unroll 1
        for (int n = 0; n < L; ++n) F[n + 1] = ((2 * n + 1) * F[n] - e) * h;
    }
}

// One thread per shell pair (i >= j): the contracted spherical blocks of
// S, T and V for every pair of contraction columns, written to both
// triangles.  Each element has one writer (no atomics).
//   S_ab = K (pi/p)^(3/2) E^x_0 E^y_0 E^z_0
//   T_ab: per axis -2 b^2 S_(i,j+2) + b (2j + 1) S_ij - j (j - 1)/2 S_(i,j-2)
//   V_ab = -sum_C Z_C K (2 pi / p) sum_tuv E^x_t E^y_u E^z_v R_tuv(P - C)
__global__ void __launch_bounds__(64) int1e_kernel(const Int1eArgs A) {
    const int64_t npair = (int64_t)A.nbas * (A.nbas + 1) / 2;
    const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= npair) return;
    int i = (int)((sqrt(8.0 * (double)k + 1.0) - 1.0) * 0.5);
    while ((int64_t)i * (i + 1) / 2 > k) --i;
    while ((int64_t)(i + 1) * (i + 2) / 2 <= k) ++i;
    const int j = (int)(k - (int64_t)i * (i + 1) / 2);
    const int la = A.sh_l[i], lb = A.sh_l[j], L = la + lb;
    const int nca = (la + 1) * (la + 2) / 2, ncb = (lb + 1) * (lb + 2) / 2;
    const int nsa = 2 * la + 1, nsb = 2 * lb + 1;
    const double* Ac = A.sh_ctr + 3 * i;
    const double* Bc = A.sh_ctr + 3 * j;
    const double ab2 = (Ac[0] - Bc[0]) * (Ac[0] - Bc[0]) +
                       (Ac[1] - Bc[1]) * (Ac[1] - Bc[1]) +
                       (Ac[2] - Bc[2]) * (Ac[2] - Bc[2]);
    const int npa = A.sh_np[i], npb = A.sh_np[j];
    const int ncta = A.sh_nc[i], nctb = A.sh_nc[j];
    const double* ea = A.exps + A.sh_eoff[i];
    const double* eb = A.exps + A.sh_eoff[j];
    const double* ca = A.coeffs + A.sh_coff[i];
    const double* cb = A.coeffs + A.sh_coff[j];
    double E[3][4 * kEJ * kET];
    double s[100], t[100], v[100], F[7], r0[7], R[84];
#pragma unroll 1
    for (int ci = 0; ci < ncta; ++ci)
#pragma unroll 1
        for (int cj = 0; cj < nctb; ++cj) {
#pragma unroll 1
            for (int q = 0; q < nca * ncb; ++q) s[q] = t[q] = v[q] = 0.0;
#pragma unroll 1
            for (int a = 0; a < npa; ++a)
#pragma unroll 1
                for (int b = 0; b < npb; ++b) {
                    const double al = ea[a], be = eb[b], p = al + be;
                    const double K = exp(-al * be / p * ab2);
                    const double cc = ca[a * ncta + ci] * cb[b * nctb + cj] * K;
                    if (cc == 0.0) continue;
                    double P[3];
#pragma unroll
                    for (int x = 0; x < 3; ++x) {
                        P[x] = (al * Ac[x] + be * Bc[x]) / p;
                        hermite1d_rt(la, lb + 2, 0.5 / p, P[x] - Ac[x], P[x] - Bc[x], E[x]);
                    }
                    const double sp = sqrt(M_PI / p);
                    const double s3 = cc * sp * sp * sp;
#pragma unroll 1
                    for (int qa = 0; qa < nca; ++qa) {
                        int ia[3];
                        cart_xyz(la, qa, ia[0], ia[1], ia[2]);
#pragma unroll 1
                        for (int qb = 0; qb < ncb; ++qb) {
                            int ib[3];
                            cart_xyz(lb, qb, ib[0], ib[1], ib[2]);
                            double s1[3], t1[3];
#pragma unroll
                            for (int x = 0; x < 3; ++x) {
                                const double* e = E[x] + ia[x] * kEJ * kET;
                                const int jb = ib[x];
                                s1[x] = e[jb * kET];
                                double r = -2.0 * be * be * e[(jb + 2) * kET] +
                                           be * (2 * jb + 1) * e[jb * kET];
                                if (jb >= 2) r -= 0.5 * jb * (jb - 1) * e[(jb - 2) * kET];
                                t1[x] = r;
                            }
                            s[qa * ncb + qb] += s3 * s1[0] * s1[1] * s1[2];
                            t[qa * ncb + qb] += s3 * (t1[0] * s1[1] * s1[2] +
                                                      s1[0] * t1[1] * s1[2] +
                                                      s1[0] * s1[1] * t1[2]);
                        }
                    }
#pragma unroll 1
                    for (int c = 0; c < A.natm; ++c) {
                        const double* C = A.nuc_xyz + 3 * c;
                        const double pc0 = P[0] - C[0], pc1 = P[1] - C[1], pc2 = P[2] - C[2];
                        boys_rt(L, p * (pc0 * pc0 + pc1 * pc1 + pc2 * pc2), A.boys, F);
                        double m2p = 1.0;
#pragma unroll 1
                        for (int n = 0; n <= L; ++n) {
                            r0[n] = m2p * F[n];
                            m2p *= -2.0 * p;
                        }
                        fill_r_rt(L, r0, pc0, pc1, pc2, R);
                        const double pre = -A.nuc_z[c] * cc * (2.0 * M_PI / p);
#pragma unroll 1
                        for (int qa = 0; qa < nca; ++qa) {
                            int ia[3];
                            cart_xyz(la, qa, ia[0], ia[1], ia[2]);
#pragma unroll 1
                            for (int qb = 0; qb < ncb; ++qb) {
                                int ib[3];
                                cart_xyz(lb, qb, ib[0], ib[1], ib[2]);
                                const double* ex = E[0] + (ia[0] * kEJ + ib[0]) * kET;
                                const double* ey = E[1] + (ia[1] * kEJ + ib[1]) * kET;
                                const double* ez = E[2] + (ia[2] * kEJ + ib[2]) * kET;
                                double sum = 0.0;
#pragma unroll 1
                                for (int tt = 0; tt <= ia[0] + ib[0]; ++tt)
#pragma unroll 1
                                    for (int uu = 0; uu <= ia[1] + ib[1]; ++uu) {
                                        const double exy = ex[tt] * ey[uu];
#pragma unroll 1
                                        for (int vv = 0; vv <= ia[2] + ib[2]; ++vv)
                                            sum += exy * ez[vv] * R[ridx_rt(L, tt, uu, vv)];
                                    }
                                v[qa * ncb + qb] += pre * sum;
                            }
                        }
                    }
                }
            // Cartesian -> spherical, stored to both triangles
            const double* c2a = c2s_of(la);
            const double* c2b = c2s_of(lb);
            const int row0 = A.sh_ao0[i] + ci * nsa, col0 = A.sh_ao0[j] + cj * nsb;
#pragma unroll 1
            for (int m = 0; m < nsa; ++m)
#pragma unroll 1
                for (int n = 0; n < nsb; ++n) {
                    double vs = 0.0, vt = 0.0, vv = 0.0;
#pragma unroll 1
                    for (int qa = 0; qa < nca; ++qa) {
                        const double wa = c2a[qa * nsa + m];
                        if (wa == 0.0) continue;
#pragma unroll 1
                        for (int qb = 0; qb < ncb; ++qb) {
                            const double w = wa * c2b[qb * nsb + n];
                            vs += w * s[qa * ncb + qb];
                            vt += w * t[qa * ncb + qb];
                            vv += w * v[qa * ncb + qb];
                        }
                    }
                    const int64_t e1 = (int64_t)(row0 + m) * A.nao + col0 + n;
                    const int64_t e2 = (int64_t)(col0 + n) * A.nao + row0 + m;
                    A.S[e1] = vs; A.S[e2] = vs;
                    A.T[e1] = vt; A.T[e2] = vt;
                    A.V[e1] = vv; A.V[e2] = vv;
                }
        }
}

cudaError_t upload_int1e_c2s(const double* all110) {
    return cudaMemcpyToSymbol(c_c2s_all, all110, sizeof(double) * 110);
}

cudaError_t launch_int1e(const Int1eArgs& a, cudaStream_t s) {
    const int64_t npair = (int64_t)a.nbas * (a.nbas + 1) / 2;
    if (npair <= 0) return cudaSuccess;
    int1e_kernel<<<(unsigned)((npair + 63) / 64), 64, 0, s>>>(a);
    return cudaGetLastError();
}

// -- Hermite densities ---------------------------------------------------------

// One thread per shell pair (la >= lb): Dc = c2s'_A^T D_AB c2s'_B in the
// Cartesian components (c2s' = the d/f transforms; identity for s and p,
// whose angular factors are folded into pref), then for each of its
// primitive pairs dh[tuv] = w pref sum_{ab} Dc_ab E^x E^y E^z, w = 2 for
// A != B (the D_BA half) and 1 for a diagonal pair.  Also the pair's
// screening factor w sum |D_AB| (FP32, rounded up).
__global__ void __launch_bounds__(64) dh_kernel(const DhArgs A) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= A.npairs) return;
    const int cls = A.pclass[k];
    int la = 0, lb = 0;
    while ((la + 1) * (la + 2) / 2 <= cls) ++la;
    lb = cls - la * (la + 1) / 2;
    const int L = la + lb, nr = (L + 1) * (L + 2) * (L + 3) / 6;
    const int nca = (la + 1) * (la + 2) / 2, ncb = (lb + 1) * (lb + 2) / 2;
    const int nsa = 2 * la + 1, nsb = 2 * lb + 1;
    int nax = 0;                                   // E entries per axis
    for (int i = 0; i <= la; ++i)
        for (int j = 0; j <= lb; ++j) nax += i + j + 1;
    const int4 h = A.hdr[k];
    const int ia0 = h.x, ib0 = h.y, pp0 = h.z, npp = h.w & 0xffff;
    const double w = ((h.w >> 16) & 1) ? 1.0 : 2.0;
    double dabs = 0.0;
#pragma unroll 1
    for (int m = 0; m < nsa; ++m)
#pragma unroll 1
        for (int n = 0; n < nsb; ++n)
            dabs += fabs(A.D[(int64_t)(ia0 + m) * A.nao + ib0 + n]);
    A.pair_dabs[k] = __double2float_ru(w * dabs * (1.0 + 1e-6));
    double Dc[100];
    const double* c2a = c2s_of(la);
    const double* c2b = c2s_of(lb);
#pragma unroll 1
    for (int qa = 0; qa < nca; ++qa)
#pragma unroll 1
        for (int qb = 0; qb < ncb; ++qb) {
            double acc = 0.0;
#pragma unroll 1
            for (int m = 0; m < nsa; ++m) {
                const double wa = la >= 2 ? c2a[qa * nsa + m] : (qa == m ? 1.0 : 0.0);
                if (wa == 0.0) continue;
#pragma unroll 1
                for (int n = 0; n < nsb; ++n) {
                    const double wb = lb >= 2 ? c2b[qb * nsb + n] : (qb == n ? 1.0 : 0.0);
                    acc += wa * wb * A.D[(int64_t)(ia0 + m) * A.nao + ib0 + n];
                }
            }
            Dc[qa * ncb + qb] = acc;
        }
    const double* Ecls = A.E + A.e_base[cls];
    const int cpp0 = A.pp_begin[cls];
    double dh[84];
#pragma unroll 1
    for (int m = pp0; m < pp0 + npp; ++m) {
        const double* e = Ecls + (int64_t)(m - cpp0) * 3 * nax;
#pragma unroll 1
        for (int q = 0; q < nr; ++q) dh[q] = 0.0;
#pragma unroll 1
        for (int qa = 0; qa < nca; ++qa) {
            int ia[3];
            cart_xyz(la, qa, ia[0], ia[1], ia[2]);
#pragma unroll 1
            for (int qb = 0; qb < ncb; ++qb) {
                const double d = Dc[qa * ncb + qb];
                if (d == 0.0) continue;
                int ib[3];
                cart_xyz(lb, qb, ib[0], ib[1], ib[2]);
                const double* ex = e + f64::eoff(lb, ia[0], ib[0]);
                const double* ey = e + nax + f64::eoff(lb, ia[1], ib[1]);
                const double* ez = e + 2 * nax + f64::eoff(lb, ia[2], ib[2]);
#pragma unroll 1
                for (int tt = 0; tt <= ia[0] + ib[0]; ++tt)
#pragma unroll 1
                    for (int uu = 0; uu <= ia[1] + ib[1]; ++uu) {
                        const double dxy = d * ex[tt] * ey[uu];
#pragma unroll 1
                        for (int vv = 0; vv <= ia[2] + ib[2]; ++vv)
                            dh[ridx_rt(L, tt, uu, vv)] += dxy * ez[vv];
                    }
            }
        }
        const double pre = w * A.pref[m];
        const int64_t off = A.dh_off[m];
#pragma unroll 1
        for (int q = 0; q < nr; ++q) {
            const double val = pre * dh[q];
            A.dh64[off + q] = val;
            A.dh32[off + q] = (float)val;
        }
    }
}

cudaError_t launch_dh(const DhArgs& a, cudaStream_t s) {
    if (a.npairs <= 0) return cudaSuccess;
    dh_kernel<<<(unsigned)((a.npairs + 63) / 64), 64, 0, s>>>(a);
    return cudaGetLastError();
}

// -- block geometry ------------------------------------------------------------

// centroid and radius (FP64, radius rounded up) of each 32-point block:
// one warp per block
__global__ void block_geom_kernel(const double* __restrict__ xyz, int64_t npts,
                                  int nblk, float4* __restrict__ cr) {
    const int blk = (int)(((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5);
    const int lane = threadIdx.x & 31;
    if (blk >= nblk) return;
    const int64_t g = (int64_t)blk * 32 + lane;
    const bool ok = g < npts;
    double x = 0, y = 0, z = 0;
    if (ok) { x = xyz[3 * g]; y = xyz[3 * g + 1]; z = xyz[3 * g + 2]; }
    double sx = x, sy = y, sz = z, cnt = ok ? 1.0 : 0.0;
    for (int o = 16; o > 0; o >>= 1) {
        sx += __shfl_xor_sync(0xffffffffu, sx, o);
        sy += __shfl_xor_sync(0xffffffffu, sy, o);
        sz += __shfl_xor_sync(0xffffffffu, sz, o);
        cnt += __shfl_xor_sync(0xffffffffu, cnt, o);
    }
    const double c0 = sx / cnt, c1 = sy / cnt, c2 = sz / cnt;
    double r = ok ? sqrt((x - c0) * (x - c0) + (y - c1) * (y - c1) + (z - c2) * (z - c2))
                  : 0.0;
    for (int o = 16; o > 0; o >>= 1) r = fmax(r, __shfl_xor_sync(0xffffffffu, r, o));
    if (lane == 0)
        cr[blk] = make_float4((float)c0, (float)c1, (float)c2,
                              __double2float_ru(r * (1.0 + 1e-7) + 1e-7));
}

// -- Hartree potential ---------------------------------------------------------

// Precision traits: FP64 (FP64 Boys table, coordinates and Hermite
// densities) or FP32 (FP32 Boys, coordinates as hi + lo, FP32 Hermite
// densities and R; each 32-pair chunk summed in FP32, then in FP64).
template<bool F64> struct HartreeTraits;
template<> struct HartreeTraits<true> {
    typedef double Real;
    static constexpr int kTabBytes = kBoys64Nodes * kBoys64Cols * 8;
};
template<> struct HartreeTraits<false> {
    typedef float Real;
    static constexpr int kTabBytes = 145 * 5 * 16;
};

template<bool F64, int L>
__device__ __forceinline__ typename HartreeTraits<F64>::Real hartree_pp(const HartreeArgs& A, const int m,
                                             const double gx, const double gy,
                                             const double gz, const float3 gh,
                                             const float3 gl, const void* stab) {
    typedef typename HartreeTraits<F64>::Real Real;
    Real px, py, pz, p;
    if constexpr (F64) {
        px = A.P[3 * m] - gx; py = A.P[3 * m + 1] - gy; pz = A.P[3 * m + 2] - gz;
        p = A.p[m];
    } else {
        const float4 hi = A.geo[2 * m], lo = A.geo[2 * m + 1];
        px = (hi.x - gh.x) + (lo.x - gl.x);
        py = (hi.y - gh.y) + (lo.y - gl.y);
        pz = (hi.z - gh.z) + (lo.z - gl.z);
        p = A.p32[m];
    }
    const Real T = p * (px * px + py * py + pz * pz);
    Real F[L + 1], r0[L + 1];
    if constexpr (F64)
        boys64<L>(T, static_cast<const double*>(stab), F);
    else
        boys_fp32<L>(T, F, static_cast<const float4*>(stab));
    Real m2p = Real(1);
#pragma unroll
    for (int n = 0; n <= L; ++n) {
        r0[n] = m2p * F[n];
        m2p *= Real(-2) * p;
    }
    const int64_t off = A.dh_off[m];
    const Real* dh;
    if constexpr (F64) dh = A.dh64 + off; else dh = A.dh32 + off;
    if constexpr (L == 0) return hermite_dot_0<Real>(r0, px, py, pz, dh);
    else if constexpr (L == 1) return hermite_dot_1<Real>(r0, px, py, pz, dh);
    else if constexpr (L == 2) return hermite_dot_2<Real>(r0, px, py, pz, dh);
    else if constexpr (L == 3) return hermite_dot_3<Real>(r0, px, py, pz, dh);
    else if constexpr (L == 4) return hermite_dot_4<Real>(r0, px, py, pz, dh);
    else if constexpr (L == 5) return hermite_dot_5<Real>(r0, px, py, pz, dh);
    else return hermite_dot_6<Real>(r0, px, py, pz, dh);
}

template<bool F64>
__device__ __forceinline__ typename HartreeTraits<F64>::Real hartree_pair(
    const HartreeArgs& A, const int L, const int pp0, const int npp, const double gx,
    const double gy, const double gz, const float3 gh, const float3 gl,
    const void* stab) {
    typename HartreeTraits<F64>::Real s = 0;
    for (int m = pp0; m < pp0 + npp; ++m) {
        switch (L) {
        case 0: s += hartree_pp<F64, 0>(A, m, gx, gy, gz, gh, gl, stab); break;
        case 1: s += hartree_pp<F64, 1>(A, m, gx, gy, gz, gh, gl, stab); break;
        case 2: s += hartree_pp<F64, 2>(A, m, gx, gy, gz, gh, gl, stab); break;
        case 3: s += hartree_pp<F64, 3>(A, m, gx, gy, gz, gh, gl, stab); break;
        case 4: s += hartree_pp<F64, 4>(A, m, gx, gy, gz, gh, gl, stab); break;
        case 5: s += hartree_pp<F64, 5>(A, m, gx, gy, gz, gh, gl, stab); break;
        default: s += hartree_pp<F64, 6>(A, m, gx, gy, gz, gh, gl, stab); break;
        }
    }
    return s;
}

// One warp per 32-point block (one point per lane), blocks taken from a
// counter.  For 32 pairs at a time each lane screens one pair (the COSX
// kernels' locked bound times w sum |D_AB|), a ballot keeps the warp on the
// kept pairs, and every lane adds the pair's primitive pairs at its point.
// The FP32 form sums each 32-pair chunk in FP32 and the chunks in FP64; the
// FP64 form sums in FP64.  Fixed order: bitwise reproducible.
template<bool F64>
__global__ void __launch_bounds__(128) hartree_kernel(const HartreeArgs A) {
    extern __shared__ float4 smem[];
    {
        const int n = HartreeTraits<F64>::kTabBytes / 16;
        const float4* src = F64 ? reinterpret_cast<const float4*>(A.boys64) : A.boys32;
        for (int i = threadIdx.x; i < n; i += blockDim.x) smem[i] = src[i];
    }
    __syncthreads();
    const void* stab = smem;
    const int lane = threadIdx.x & 31;
    unsigned long long kept = 0;
    for (;;) {
        int blk = 0;
        if (lane == 0) blk = atomicAdd(A.work, 1);
        blk = __shfl_sync(0xffffffffu, blk, 0);
        if (blk >= A.nblk) break;
        const int64_t g0 = (int64_t)blk * 32 + lane;
        const bool ok = g0 < A.npts;
        const int64_t g = ok ? g0 : A.npts - 1;
        const double gx = A.coords[3 * g], gy = A.coords[3 * g + 1], gz = A.coords[3 * g + 2];
        float3 gh = make_float3(0.f, 0.f, 0.f), gl = gh;
        if (!F64) {
            gh = make_float3((float)gx, (float)gy, (float)gz);
            gl = make_float3((float)(gx - (double)gh.x), (float)(gy - (double)gh.y),
                             (float)(gz - (double)gh.z));
        }
        const float4 cr = A.blk_cr[blk];
        double v = 0.0;
        for (int c0 = 0; c0 < A.npairs; c0 += 32) {
            const int k = c0 + lane;
            bool keep = k < A.npairs;
            int4 h = make_int4(0, 0, 0, 0);
            if (keep) {
                h = A.hdr[k];
                if (A.tol > 0.0f)
                    keep = screen_pair(A.tol, A.bnd, A.bpref, cr, h, A.ptau[k],
                                       A.pair_dabs[k]);
            }
            unsigned mask = __ballot_sync(0xffffffffu, keep);
            kept += __popc(mask);
            typename HartreeTraits<F64>::Real chunk = 0;
            while (mask) {
                const int src = __ffs(mask) - 1;
                mask &= mask - 1;
                const int kk = c0 + src;
                const int pp0 = __shfl_sync(0xffffffffu, h.z, src);
                const int npp = __shfl_sync(0xffffffffu, h.w, src) & 0xffff;
                const int L = A.pair_L[kk];
                chunk += hartree_pair<F64>(A, L, pp0, npp, gx, gy, gz, gh, gl, stab);
            }
            v += (double)chunk;
        }
        if (ok) A.v[g0] = v;
    }
    if (lane == 0 && A.kept) atomicAdd(A.kept, kept);
}

cudaError_t launch_block_geom(const double* xyz, int64_t npts, int nblk, float4* cr,
                              cudaStream_t s) {
    if (nblk <= 0) return cudaSuccess;
    block_geom_kernel<<<(unsigned)((nblk * 32 + 127) / 128), 128, 0, s>>>(xyz, npts,
                                                                          nblk, cr);
    return cudaGetLastError();
}

// One point per lane.  A two-point form (the pair's data read once for
// both points, each point keeping its own sub-block's screen: bitwise the
// same values) measured slower in the device SCF (J 0.250 against
// 0.234 s on 8 waters): its extra registers cost more occupancy than the
// shared loads saved.
cudaError_t launch_hartree(const HartreeArgs& a, bool fp64, cudaStream_t s) {
    if (a.nblk <= 0) return cudaSuccess;
    const int grid = std::max(1, std::min(a.nblk / 4 + 1, sm_count() * 8));
    if (fp64) {
        const size_t smem = HartreeTraits<true>::kTabBytes;
        cudaError_t e = cudaFuncSetAttribute(hartree_kernel<true>,
                                             cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)smem);
        if (e != cudaSuccess) return e;
        hartree_kernel<true><<<grid, 128, smem, s>>>(a);
    } else {
        hartree_kernel<false><<<grid, 128, HartreeTraits<false>::kTabBytes, s>>>(a);
    }
    return cudaGetLastError();
}

}  // namespace scf
}  // namespace wb
