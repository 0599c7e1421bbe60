// Supporting kernels of the COSX K build: per-omega primitive constants,
// grid coordinate split, sub-block statistics for the screen, FP64 AO
// evaluation, precision casts, the dense validation kernel and the Boys
// batch kernel.
#include <cmath>

#include "boys.cuh"
#include "launch.hpp"
#include "screen.cuh"

namespace wb {

// -- per-omega primitive-pair constants (gpu/sgx_k.py:783-811) --------------
// theta = w^2 / (w^2 + p) (1 for w = 0), tp = theta p and the R000
// coefficients c_n = pref sqrt(theta) (-2 p theta)^n, n = 0..6, formed in
// FP64 (IEEE-rounded, so identical to a host evaluation) and stored as FP32
// hi + lo.  pref already carries C_a C_b K_AB 2 pi / p and the s/p
// spherical normalisation.
__global__ void omega_kernel(int npp, const double* __restrict__ p,
                             const double* __restrict__ pref, double omega,
                             float4* __restrict__ om) {
    const int m = blockIdx.x * blockDim.x + threadIdx.x;
    if (m >= npp) return;
    const double pm = p[m];
    double th = 1.0, sth = 1.0;
    if (omega > 0.0) {
        const double w2 = omega * omega;
        th = w2 / (w2 + pm);
        sth = sqrt(th);
    }
    const double tp = th * pm;
    const double q = -2.0 * pm * th;
    float rec[20];
    rec[0] = (float)tp;
    rec[1] = (float)(tp - (double)rec[0]);
    double c = pref[m] * sth;
    // far field (T = tp r^2 >= 36, erf(sqrt T) = 1 in FP64): R000_n =
    // (-1)^n (2n-1)!! K0 r^-(2n+1) with K0 = c_0 sqrt(pi) / (2 sqrt(tp))
    const double k0 = c * 0.88622692545275801365 / sqrt(tp);
    for (int n = 0; n < 7; ++n) {
        const float hi = (float)c;
        rec[2 + 2 * n] = hi;
        rec[3 + 2 * n] = (float)(c - (double)hi);
        c *= q;
    }
    rec[16] = (float)k0;
    rec[17] = (float)(k0 - (double)rec[16]);
    rec[18] = (float)(36.0 / tp);            // r^2 at which T reaches 36
    rec[19] = 0.0f;
    float4* o = om + 5 * (long long)m;
    o[0] = make_float4(rec[0], rec[1], rec[2], rec[3]);
    o[1] = make_float4(rec[4], rec[5], rec[6], rec[7]);
    o[2] = make_float4(rec[8], rec[9], rec[10], rec[11]);
    o[3] = make_float4(rec[12], rec[13], rec[14], rec[15]);
    o[4] = make_float4(rec[16], rec[17], rec[18], rec[19]);
}

cudaError_t launch_omega(int npp, const double* p, const double* pref,
                         double omega, float4* om, cudaStream_t s) {
    if (npp <= 0) return cudaSuccess;
    omega_kernel<<<(npp + 255) / 256, 256, 0, s>>>(npp, p, pref, omega, om);
    return cudaGetLastError();
}

// Packed per-class primitive-pair records for the class kernels: one
// contiguous record per pair (P hi, P lo, the first n_om float4 of the
// omega record, the Hermite E block) so that a pair is one base address.
__global__ void pack_records_kernel(const RecPack P, int npp,
                                    const float4* __restrict__ geo,
                                    const float4* __restrict__ om,
                                    const float4* __restrict__ E,
                                    float4* __restrict__ rec) {
    const int m = blockIdx.x * blockDim.x + threadIdx.x;
    if (m >= npp) return;
    int c = 0;
    while (c < 9 && m >= P.pp_end[c]) ++c;
    if (m < P.pp_begin[c] || m >= P.pp_end[c]) return;
    const int ml = m - P.pp_begin[c];
    float4* r = rec + P.rec_off[c] + (long long)ml * P.stride[c];
    r[0] = geo[2 * (long long)m];
    r[1] = geo[2 * (long long)m + 1];
    // omega record: its first n_om - 1 float4 (theta p, c_n), then the
    // far-field float4 (K0 hi, K0 lo, r^2 threshold)
    for (int q = 0; q + 1 < P.nom[c]; ++q) r[2 + q] = om[5 * (long long)m + q];
    r[1 + P.nom[c]] = om[5 * (long long)m + 4];
    const float4* e = E + P.e_off[c] + (long long)ml * P.ne[c];
    for (int q = 0; q < P.ne[c]; ++q) r[2 + P.nom[c] + q] = e[q];
}

cudaError_t launch_pack_records(const RecPack& P, int npp, const float4* geo,
                                const float4* om, const float4* E,
                                float4* rec, cudaStream_t s) {
    if (npp <= 0) return cudaSuccess;
    pack_records_kernel<<<(npp + 127) / 128, 128, 0, s>>>(P, npp, geo, om, E, rec);
    return cudaGetLastError();
}

__global__ void pack_records2_kernel(const RecPack P, int npp,
                                     const float4* __restrict__ geo,
                                     const float4* __restrict__ oma,
                                     const float4* __restrict__ omb,
                                     const float4* __restrict__ E,
                                     float4* __restrict__ rec) {
    const int m = blockIdx.x * blockDim.x + threadIdx.x;
    if (m >= npp) return;
    int c = 0;
    while (c < 9 && m >= P.pp_end[c]) ++c;
    if (m < P.pp_begin[c] || m >= P.pp_end[c]) return;
    const int ml = m - P.pp_begin[c];
    const int nom = P.nom[c];
    float4* r = rec + P.rec_off[c] + (long long)ml * P.stride[c];
    r[0] = geo[2 * (long long)m];
    r[1] = geo[2 * (long long)m + 1];
    const float4* om[2] = {oma, omb};
    for (int w = 0; w < 2; ++w) {
        for (int q = 0; q + 1 < nom; ++q) r[2 + w * nom + q] = om[w][5 * (long long)m + q];
        r[1 + (w + 1) * nom] = om[w][5 * (long long)m + 4];
    }
    const float4* e = E + P.e_off[c] + (long long)ml * P.ne[c];
    for (int q = 0; q < P.ne[c]; ++q) r[2 + 2 * nom + q] = e[q];
}

cudaError_t launch_pack_records2(const RecPack& P, int npp, const float4* geo,
                                 const float4* om_a, const float4* om_b,
                                 const float4* E, float4* rec, cudaStream_t s) {
    if (npp <= 0) return cudaSuccess;
    pack_records2_kernel<<<(npp + 127) / 128, 128, 0, s>>>(P, npp, geo, om_a, om_b,
                                                         E, rec);
    return cudaGetLastError();
}

// -- FP64 (npts, 3) -> FP32 SoA hi / lo, padded with zeros to ld ----------
__global__ void grid_prep_kernel(const double* __restrict__ c, int64_t npts,
                                 int64_t ld, float* __restrict__ hi,
                                 float* __restrict__ lo) {
    const int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= ld) return;
    for (int x = 0; x < 3; ++x) {
        float h = 0.0f, l = 0.0f;
        if (g < npts) {
            const double v = c[g * 3 + x];
            h = (float)v;
            l = (float)(v - (double)h);
        }
        hi[x * ld + g] = h;
        lo[x * ld + g] = l;
    }
}

cudaError_t launch_grid_prep(const double* coords, int64_t npts, int64_t ld,
                             float* hi, float* lo, cudaStream_t s) {
    if (ld <= 0) return cudaSuccess;
    grid_prep_kernel<<<(unsigned)((ld + 255) / 256), 256, 0, s>>>(coords, npts,
                                                                  ld, hi, lo);
    return cudaGetLastError();
}

// -- sub-block statistics (gpu/sgx_k.py:866-903) ---------------------------
// One warp per 128-point block (four points per lane): for its 32-point
// quarters (the reference's sub-block size), its 64-point halves and the
// whole block, the FP64 centroid and radius of the valid points (centroid
// rounded to nearest FP32, radius rounded up) and, for every (virtual)
// shell, msh = max_g fl32(w_g) sum_{t in shell} |F_tg|.  One pass over F
// serves the 32-, 64- and 128-point class kernels.  Block b of size 32 * 2^k
// covers points [b 32 2^k, (b + 1) 32 2^k); blocks past ld are not written.
__device__ __forceinline__ double warp_sum_d(double v) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}
__device__ __forceinline__ double warp_max_d(double v) {
    for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}
__device__ __forceinline__ float4 centroid_radius(const double* sum, int n,
                                                  double d) {
    float r = (float)d;
    if ((double)r < d) r = nextafterf(r, INFINITY);
    if (n <= 0) return make_float4(0.0f, 0.0f, 0.0f, r);
    return make_float4((float)(sum[0] / n), (float)(sum[1] / n),
                       (float)(sum[2] / n), r);
}

__global__ void sub_stats_kernel(const BlockStatsOut O,
                                 const double* __restrict__ coords,
                                 const double* __restrict__ w,
                                 const float* __restrict__ F, int64_t npts,
                                 int64_t ld, int nvshell,
                                 const int* __restrict__ vs_ao0,
                                 const int* __restrict__ vs_nf) {
    const int blk = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    const int nblk128 = (int)((ld + 127) / 128);
    if (blk >= nblk128) return;
    // blocks of each level that exist: 32 * 2^k points starting inside ld
    int64_t g[4];
    bool valid[4];
    double c[4][3];
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        g[q] = (int64_t)blk * 128 + 32 * q + lane;
        valid[q] = g[q] < npts;
        for (int x = 0; x < 3; ++x) c[q][x] = valid[q] ? coords[g[q] * 3 + x] : 0.0;
    }
    int nv[4];
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        const int64_t rem = npts - ((int64_t)blk * 128 + 32 * q);
        nv[q] = rem >= 32 ? 32 : (rem > 0 ? (int)rem : 0);
    }
    double s[4][3];
#pragma unroll
    for (int q = 0; q < 4; ++q)
        for (int x = 0; x < 3; ++x) s[q][x] = warp_sum_d(c[q][x]);
    // level k = 0, 1, 2: block j of the level covers quarters [j 2^k, (j+1) 2^k)
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        const int span = 1 << k;
#pragma unroll
        for (int j = 0; j < 4 / span; ++j) {
            double sum[3] = {0.0, 0.0, 0.0};
            int n = 0;
            for (int q = j * span; q < (j + 1) * span; ++q) {
                for (int x = 0; x < 3; ++x) sum[x] += s[q][x];
                n += nv[q];
            }
            double m[3];
            for (int x = 0; x < 3; ++x) m[x] = n ? sum[x] / n : 0.0;
            double d = 0.0;
            for (int q = j * span; q < (j + 1) * span; ++q) {
                if (!valid[q]) continue;
                double e2 = 0.0;
                for (int x = 0; x < 3; ++x) {
                    const double e = c[q][x] - m[x];
                    e2 += e * e;
                }
                d = fmax(d, sqrt(e2));
            }
            d = warp_max_d(d);
            const int64_t b = (int64_t)blk * (4 / span) + j;
            if (lane == 0 && b * 32 * span < ld) O.cr[k][b] = centroid_radius(sum, n, d);
        }
    }
    float wq[4];
#pragma unroll
    for (int q = 0; q < 4; ++q) wq[q] = valid[q] ? (float)w[g[q]] : 0.0f;
    for (int sh = 0; sh < nvshell; ++sh) {
        const int a0 = vs_ao0[sh], nf = vs_nf[sh];
        float acc[4] = {0.0f, 0.0f, 0.0f, 0.0f};
        for (int t = 0; t < nf; ++t) {
            const int64_t row = (int64_t)(a0 + t) * ld;
#pragma unroll
            for (int q = 0; q < 4; ++q)
                if (valid[q]) acc[q] += fabsf(F[row + g[q]]) * wq[q];
        }
#pragma unroll
        for (int q = 0; q < 4; ++q)
            for (int o = 16; o > 0; o >>= 1)
                acc[q] = fmaxf(acc[q], __shfl_xor_sync(0xffffffffu, acc[q], o));
        if (lane == 0) {
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                const int64_t b = (int64_t)blk * 4 + q;
                if (b * 32 < ld) O.msh[0][b * nvshell + sh] = acc[q];
            }
#pragma unroll
            for (int j = 0; j < 2; ++j) {
                const int64_t b = (int64_t)blk * 2 + j;
                if (b * 64 < ld)
                    O.msh[1][b * nvshell + sh] = fmaxf(acc[2 * j], acc[2 * j + 1]);
            }
            O.msh[2][(int64_t)blk * nvshell + sh] =
                fmaxf(fmaxf(acc[0], acc[1]), fmaxf(acc[2], acc[3]));
        }
    }
}

cudaError_t launch_sub_stats(const double* coords, const double* weights,
                             const float* F, int64_t npts, int64_t ld,
                             int nvshell, const int* vs_ao0, const int* vs_nf,
                             const BlockStatsOut& out, cudaStream_t s) {
    const int64_t nblk = (ld + 127) / 128;
    if (nblk <= 0) return cudaSuccess;
    const int warps = 4;
    sub_stats_kernel<<<(unsigned)((nblk + warps - 1) / warps), 32 * warps, 0, s>>>(
        out, coords, weights, F, npts, ld, nvshell, vs_ao0, vs_nf);
    return cudaGetLastError();
}

// -- casts ---------------------------------------------------------------
__global__ void f64_to_f32_kernel(const double* __restrict__ in,
                                  float* __restrict__ out, int64_t n) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x)
        out[i] = __double2float_rn(in[i]);
}

cudaError_t launch_f64_to_f32(const double* in, float* out, int64_t n,
                              cudaStream_t s) {
    if (n <= 0) return cudaSuccess;
    const int64_t blocks = grid_stride_blocks(n, 256, 64);
    f64_to_f32_kernel<<<(unsigned)blocks, 256, 0, s>>>(in, out, n);
    return cudaGetLastError();
}

// out[mu, g] = w_g * (double) G[mu, g]  (gpu/sgx_k.py:734: FP64 weights)
__global__ void weight_g_kernel(const float* __restrict__ G,
                                const double* __restrict__ w, int64_t npts,
                                int64_t ld, int64_t total,
                                double* __restrict__ out) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < total;
         i += (int64_t)gridDim.x * blockDim.x) {
        const int64_t g = i % ld;
        out[i] = g < npts ? w[g] * (double)G[i] : 0.0;
    }
}

cudaError_t launch_weight_g(const float* G, const double* w, int64_t npts,
                            int64_t ld, int nao, double* out, cudaStream_t s) {
    const int64_t total = ld * nao;
    if (total <= 0) return cudaSuccess;
    const int64_t blocks = grid_stride_blocks(total, 256, 64);
    weight_g_kernel<<<(unsigned)blocks, 256, 0, s>>>(G, w, npts, ld, total, out);
    return cudaGetLastError();
}

// G[mu, g] = sum of the class partial-G rows src[mu] (ascending class
// order, -1 = none): the fixed-order combination of the concurrently
// filled class buffers.  Four points per thread (ld is a multiple of 32).
__global__ void gsum_kernel(const float* __restrict__ gc,
                            const int4* __restrict__ src, int64_t ld,
                            float* __restrict__ G) {
    const int mu = blockIdx.y;
    const int64_t i = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) * 4;
    if (i >= ld) return;
    const int4 sr = src[mu];
    const int rows[4] = {sr.x, sr.y, sr.z, sr.w};
    float4 acc = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        if (rows[j] < 0) continue;
        const float4 v = *reinterpret_cast<const float4*>(gc + rows[j] * ld + i);
        acc.x += v.x; acc.y += v.y; acc.z += v.z; acc.w += v.w;
    }
    *reinterpret_cast<float4*>(G + (int64_t)mu * ld + i) = acc;
}

// the same over two buffer sets (the two halves of split blocks): the
// first set's rows, then the second's, in fixed order
__global__ void gsum2_kernel(const float* __restrict__ gc0,
                             const float* __restrict__ gc1,
                             const int4* __restrict__ src, int64_t ld,
                             float* __restrict__ G) {
    const int mu = blockIdx.y;
    const int64_t i = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) * 4;
    if (i >= ld) return;
    const int4 sr = src[mu];
    const int rows[4] = {sr.x, sr.y, sr.z, sr.w};
    float4 acc = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    for (int h = 0; h < 2; ++h) {
        const float* gc = h ? gc1 : gc0;
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            if (rows[j] < 0) continue;
            const float4 v = *reinterpret_cast<const float4*>(gc + rows[j] * ld + i);
            acc.x += v.x; acc.y += v.y; acc.z += v.z; acc.w += v.w;
        }
    }
    *reinterpret_cast<float4*>(G + (int64_t)mu * ld + i) = acc;
}

// Longest-processing-time order of the point blocks of each class (one
// CTA per class): a counting sort of the blocks by their measured cost in
// 2^(1/8) steps, costliest first.  Each kernel hands its blocks out in this
// order, so the last blocks taken -- the tail of the launch -- are the
// cheap ones.  Within a step the order is arbitrary; results do not depend
// on it (a block's G columns are written by one warp in fixed pair order).
__global__ void block_order_kernel(const BlockOrderArgs P) {
    const int c = blockIdx.x;
    const int n = P.n[c];
    if (n <= 0) return;
    const float* __restrict__ cost = P.cost + (long long)c * P.stride;
    int* __restrict__ order = P.order + (long long)c * P.stride;
    __shared__ unsigned cnt[256];
    for (int b = threadIdx.x; b < 256; b += blockDim.x) cnt[b] = 0u;
    __syncthreads();
    auto bucket = [](float x) {
        // 255 - 8 log2(1 + cost), clamped: bucket 0 holds the costliest
        const float l = 8.0f * __log2f(1.0f + fmaxf(x, 0.0f));
        const int b = 255 - (int)fminf(l, 255.0f);
        return b < 0 ? 0 : b;
    };
    for (int i = threadIdx.x; i < n; i += blockDim.x)
        atomicAdd(&cnt[bucket(cost[i])], 1u);
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned run = 0;
        for (int b = 0; b < 256; ++b) {
            const unsigned t = cnt[b];
            cnt[b] = run;
            run += t;
        }
    }
    __syncthreads();
    for (int i = threadIdx.x; i < n; i += blockDim.x)
        order[atomicAdd(&cnt[bucket(cost[i])], 1u)] = i;
}

cudaError_t launch_block_order(const BlockOrderArgs& P, cudaStream_t s) {
    block_order_kernel<<<kClasses, 1024, 0, s>>>(P);
    return cudaGetLastError();
}

// -- semilocal XC flow (reference gpu/xc.py:130-201) -------------------------
// Density parameters at every point: rho = sum_mu T0 X0, grad_d = 2 sum_mu
// T0 X_d and, for MGGA, tau = 1/2 sum_d sum_mu T_d X_d, with X (4, nao, ld)
// the FP64 AO values and gradients and T (1 or 4, nao, ld) = fl32(D^T X_d)
// from the FP64-accurate F GEMM.  Products in FP32 (the reference's flow is
// FP32 throughout), summed in FP32 over 8 AOs and in FP64 across groups.
// One thread per point, rows read coalesced.  Points at or past npts: 0.
__global__ void xc_rho_kernel(const double* __restrict__ X,
                              const float* __restrict__ T, int nao, int64_t ld,
                              int64_t npts, int mgga, double* __restrict__ rho) {
    const int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= ld) return;
    double acc[5] = {0.0, 0.0, 0.0, 0.0, 0.0};
    if (g < npts) {
        const int64_t pl = (int64_t)nao * ld;
        for (int m0 = 0; m0 < nao; m0 += 8) {
            float part[5] = {0.0f, 0.0f, 0.0f, 0.0f, 0.0f};
            const int m1 = min(nao, m0 + 8);
            for (int mu = m0; mu < m1; ++mu) {
                const int64_t o = (int64_t)mu * ld + g;
                const float t0 = T[o];
                part[0] = fmaf(t0, (float)X[o], part[0]);
                part[1] = fmaf(t0, (float)X[pl + o], part[1]);
                part[2] = fmaf(t0, (float)X[2 * pl + o], part[2]);
                part[3] = fmaf(t0, (float)X[3 * pl + o], part[3]);
                if (mgga) {
                    part[4] = fmaf(T[pl + o], (float)X[pl + o], part[4]);
                    part[4] = fmaf(T[2 * pl + o], (float)X[2 * pl + o], part[4]);
                    part[4] = fmaf(T[3 * pl + o], (float)X[3 * pl + o], part[4]);
                }
            }
#pragma unroll
            for (int k = 0; k < 5; ++k) acc[k] += (double)part[k];
        }
    }
    rho[g] = acc[0];
    rho[ld + g] = 2.0 * acc[1];
    rho[2 * ld + g] = 2.0 * acc[2];
    rho[3 * ld + g] = 2.0 * acc[3];
    rho[4 * ld + g] = 0.5 * acc[4];
}

cudaError_t launch_xc_rho(const double* X, const float* T, int nao, int64_t ld,
                          int64_t npts, int mgga, double* rho, cudaStream_t s) {
    if (ld <= 0) return cudaSuccess;
    xc_rho_kernel<<<(unsigned)((ld + 255) / 256), 256, 0, s>>>(X, T, nao, ld, npts,
                                                              mgga, rho);
    return cudaGetLastError();
}

// The Fock-side planes, FP32 (nao, ld) each: G0 = 1/2 v0 X0 + sum_d v_d X_d
// (the reference's aow without the weights, which the K GEMM applies) and,
// for MGGA, G_d = 1/2 vtau X_d (d = x, y, z); v (5, ld) FP64 are the
// density-parameter derivatives (chain rule applied).  Points at or past
// npts: 0.
__global__ void xc_aow_kernel(const double* __restrict__ X,
                              const double* __restrict__ v, int nao, int64_t ld,
                              int64_t npts, int mgga, float* __restrict__ G) {
    const int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int mu = blockIdx.y;
    if (g >= ld) return;
    const int64_t pl = (int64_t)nao * ld;
    const int64_t o = (int64_t)mu * ld + g;
    float g0 = 0.0f, gt[3] = {0.0f, 0.0f, 0.0f};
    if (g < npts) {
        const float u0 = (float)(0.5 * v[g]);
        g0 = u0 * (float)X[o];
#pragma unroll
        for (int d = 1; d < 4; ++d)
            g0 = fmaf((float)v[d * ld + g], (float)X[d * pl + o], g0);
        if (mgga) {
            const float ut = (float)(0.5 * v[4 * ld + g]);
#pragma unroll
            for (int d = 1; d < 4; ++d) gt[d - 1] = ut * (float)X[d * pl + o];
        }
    }
    G[o] = g0;
    if (mgga) {
#pragma unroll
        for (int d = 1; d < 4; ++d) G[d * pl + o] = gt[d - 1];
    }
}

cudaError_t launch_xc_aow(const double* X, const double* v, int nao, int64_t ld,
                          int64_t npts, int mgga, float* G, cudaStream_t s) {
    if (ld <= 0 || nao <= 0) return cudaSuccess;
    dim3 grid((unsigned)((ld + 255) / 256), (unsigned)nao);
    xc_aow_kernel<<<grid, 256, 0, s>>>(X, v, nao, ld, npts, mgga, G);
    return cudaGetLastError();
}

cudaError_t launch_gsum(const float* gc, const int4* src, int nao, int64_t ld,
                        float* G, cudaStream_t s) {
    if (nao <= 0 || ld <= 0) return cudaSuccess;
    const int64_t quads = ld / 4;
    dim3 grid((unsigned)((quads + 255) / 256), (unsigned)nao);
    gsum_kernel<<<grid, 256, 0, s>>>(gc, src, ld, G);
    return cudaGetLastError();
}

cudaError_t launch_gsum2(const float* gc0, const float* gc1, const int4* src, int nao,
                         int64_t ld, float* G, cudaStream_t s) {
    const int64_t quads = ld / 4;
    dim3 grid((unsigned)((quads + 255) / 256), (unsigned)nao);
    gsum2_kernel<<<grid, 256, 0, s>>>(gc0, gc1, src, ld, G);
    return cudaGetLastError();
}

// -- FP64 AO evaluation (gpu/ao_eval.py:255-329, deriv 0) -------------------
// One thread per (point, shell), threads of a block on consecutive points:
// every AO column is written coalesced.  d = r - A in FP64, exp in FP64,
// contraction, Cartesian monomials, cart -> sph with FP64 constants.
__constant__ double c_c2s0[1];
__constant__ double c_c2s1[9];
__constant__ double c_c2s2[30];
__constant__ double c_c2s3[70];

template<int L>
__device__ __forceinline__ const double* c2s_ptr() {
    if constexpr (L == 0) return c_c2s0;
    else if constexpr (L == 1) return c_c2s1;
    else if constexpr (L == 2) return c_c2s2;
    else return c_c2s3;
}

// exp(-a) for 0 <= a < 70 in FP64, table-driven after P. T. P. Tang,
// "Table-driven implementation of the exponential function in IEEE
// floating-point arithmetic", ACM TOMS 15 (1989) 144-157:
//   a = n ln2/64 + r, n = rint(64 a / ln2), |r| <= ln2/128, r from a
//   two-constant (Cody-Waite) reduction with n C1 exact (C1 has 40
//   significant bits, n <= 6464);
//   exp(-a) = 2^-(n >> 6) 2^-((n & 63)/64) exp(-r), the middle factor from
//   a 64-entry table, exp(-r) by its degree-5 Taylor polynomial (truncation
//   below 4e-17), the power of two applied to the exponent field.
// About 2 ulp; the AO values feed 42-bit splits.
__constant__ double c_exp2m[64];            // 2^(-j/64), j = 0..63

__device__ __forceinline__ double exp_neg(const double a,
                                          const double* __restrict__ tab) {
    const double C1 = 0.010830424696237628;     // ln2/64, high 40 bits
    const double C2 = 1.1517191508074686e-14;   // ln2/64 - C1
    const double t = a * 92.33248261689366;      // 64 / ln2
    const int n = __double2int_rn(t);
    const double dn = (double)n;
    double r = fma(-dn, C1, a);
    r = fma(-dn, C2, r);
    const double x = -r;
    double p = fma(x, 1.0 / 120.0, 1.0 / 24.0);
    p = fma(x, p, 1.0 / 6.0);
    p = fma(x, p, 0.5);
    p = fma(x, p, 1.0);
    p = fma(x, p, 1.0);
    // 2^-(n >> 6) 2^-(j/64): subtract from the table entry's exponent field
    const double tj = tab[n & 63];
    const long long bits = __double_as_longlong(tj) - ((long long)(n >> 6) << 52);
    return __longlong_as_double(bits) * p;
}

__device__ __forceinline__ double ipow(double x, int n) {
    double r = 1.0;
    for (int i = 0; i < n; ++i) r *= x;
    return r;
}

template<int L>
__device__ __forceinline__ void ao_shell(const AoArgs& A, int sh, int64_t g,
                                         double dx, double dy, double dz,
                                         double r2, const double* etab) {
    constexpr int NC = (L + 1) * (L + 2) / 2, NS = 2 * L + 1;
    const double* c2s = c2s_ptr<L>();
    const int np = A.sh_np[sh], nc = A.sh_nc[sh];
    const double* ex = A.exps + A.sh_eoff[sh];
    const double* co = A.coeffs + A.sh_coff[sh];
    const int ao0 = A.sh_ao0[sh];
    // the spherical angular factors, formed on the first contraction with a
    // nonzero radial part: at most points of a cluster every primitive of a
    // shell is below exp(-70), and the FP64 angular work is skipped there
    double ang[NS];
    bool have_ang = false;
    for (int ci = 0; ci < nc; ++ci) {
        double rad = 0.0;
        for (int k = 0; k < np; ++k) {
            // exp(-70) ~ 4e-31: such a primitive is zero at FP64 parity with
            // any AO value of order one; skipping it avoids the FP64 exp
            const double a = ex[k] * r2;
            if (a < 70.0) rad += co[k * nc + ci] * exp_neg(a, etab);
        }
        if (rad == 0.0) {
#pragma unroll
            for (int m = 0; m < NS; ++m) A.X[(int64_t)(ao0 + ci * NS + m) * A.ld + g] = 0.0;
            continue;
        }
        if (!have_ang) {
            double mono[NC];
            int c = 0;
#pragma unroll
            for (int lx = L; lx >= 0; --lx)
#pragma unroll
                for (int ly = L - lx; ly >= 0; --ly)
                    mono[c++] = ipow(dx, lx) * ipow(dy, ly) * ipow(dz, L - lx - ly);
#pragma unroll
            for (int m = 0; m < NS; ++m) {
                double v = 0.0;
#pragma unroll
                for (int q = 0; q < NC; ++q) v += c2s[q * NS + m] * mono[q];
                ang[m] = v;
            }
            have_ang = true;
        }
#pragma unroll
        for (int m = 0; m < NS; ++m)
            A.X[(int64_t)(ao0 + ci * NS + m) * A.ld + g] = rad * ang[m];
    }
}

__global__ void ao_eval_kernel(const AoArgs A) {
    __shared__ double etab[64];
    if (threadIdx.x < 64) etab[threadIdx.x] = c_exp2m[threadIdx.x];
    __syncthreads();
    const int sh = blockIdx.y;
    const int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= A.ld) return;
    const int l = A.sh_l[sh];
    if (g >= A.npts) {
        const int n = A.sh_nc[sh] * (2 * l + 1);
        for (int i = 0; i < n; ++i) A.X[(int64_t)(A.sh_ao0[sh] + i) * A.ld + g] = 0.0;
        return;
    }
    const double dx = A.coords[g * 3] - A.sh_ctr[sh * 3];
    const double dy = A.coords[g * 3 + 1] - A.sh_ctr[sh * 3 + 1];
    const double dz = A.coords[g * 3 + 2] - A.sh_ctr[sh * 3 + 2];
    const double r2 = dx * dx + dy * dy + dz * dz;
    switch (l) {
    case 0: ao_shell<0>(A, sh, g, dx, dy, dz, r2, etab); break;
    case 1: ao_shell<1>(A, sh, g, dx, dy, dz, r2, etab); break;
    case 2: ao_shell<2>(A, sh, g, dx, dy, dz, r2, etab); break;
    default: ao_shell<3>(A, sh, g, dx, dy, dz, r2, etab); break;
    }
}

// deriv 1: value and x, y, z gradients, X (4, nao, ld).  For a primitive
// x^i y^j z^k exp(-a r^2): d/dx = (i x^(i-1) - 2 a x^(i+1)) y^j z^k exp(-a r^2)
// (gpu/ao_eval.py:305-319); contracted radial sums rad0 = sum c e,
// rad1 = sum c (-2 a) e.
template<int L>
__device__ __forceinline__ void ao_shell_d1(const AoArgs& A, int sh, int64_t g,
                                            double dx, double dy, double dz,
                                            double r2, const double* etab) {
    constexpr int NC = (L + 1) * (L + 2) / 2, NS = 2 * L + 1;
    double px[L + 2], py[L + 2], pz[L + 2];
    px[0] = py[0] = pz[0] = 1.0;
#pragma unroll
    for (int e = 1; e < L + 2; ++e) {
        px[e] = px[e - 1] * dx; py[e] = py[e - 1] * dy; pz[e] = pz[e - 1] * dz;
    }
    const double* c2s = c2s_ptr<L>();
    const int np = A.sh_np[sh], nc = A.sh_nc[sh];
    const double* ex = A.exps + A.sh_eoff[sh];
    const double* co = A.coeffs + A.sh_coff[sh];
    const int ao0 = A.sh_ao0[sh];
    const int64_t plane = (int64_t)A.nao * A.ld;
    for (int ci = 0; ci < nc; ++ci) {
        double rad0 = 0.0, rad1 = 0.0;
        for (int k = 0; k < np; ++k) {
            const double a = ex[k] * r2;
            if (a >= 70.0) continue;          // below ~1e-30, see ao_shell
            const double e = co[k * nc + ci] * exp_neg(a, etab);
            rad0 += e;
            rad1 += -2.0 * ex[k] * e;
        }
        if (rad0 == 0.0 && rad1 == 0.0) {     // every primitive skipped
#pragma unroll
            for (int m = 0; m < NS; ++m) {
                const int64_t o = (int64_t)(ao0 + ci * NS + m) * A.ld + g;
                A.X[o] = 0.0;
                A.X[plane + o] = 0.0;
                A.X[2 * plane + o] = 0.0;
                A.X[3 * plane + o] = 0.0;
            }
            continue;
        }
        double cv[NC], cgx[NC], cgy[NC], cgz[NC];
        {
            int c = 0;
#pragma unroll
            for (int lx = L; lx >= 0; --lx)
#pragma unroll
                for (int ly = L - lx; ly >= 0; --ly) {
                    const int lz = L - lx - ly;
                    const double m = px[lx] * py[ly] * pz[lz];
                    cv[c] = rad0 * m;
                    cgx[c] = rad1 * px[lx + 1] * py[ly] * pz[lz] +
                             (lx ? rad0 * lx * px[lx - 1] * py[ly] * pz[lz] : 0.0);
                    cgy[c] = rad1 * px[lx] * py[ly + 1] * pz[lz] +
                             (ly ? rad0 * ly * px[lx] * py[ly - 1] * pz[lz] : 0.0);
                    cgz[c] = rad1 * px[lx] * py[ly] * pz[lz + 1] +
                             (lz ? rad0 * lz * px[lx] * py[ly] * pz[lz - 1] : 0.0);
                    ++c;
                }
        }
#pragma unroll
        for (int m = 0; m < NS; ++m) {
            double v = 0.0, gx = 0.0, gy = 0.0, gz = 0.0;
#pragma unroll
            for (int c = 0; c < NC; ++c) {
                const double t = c2s[c * NS + m];
                v += t * cv[c]; gx += t * cgx[c]; gy += t * cgy[c]; gz += t * cgz[c];
            }
            const int64_t o = (int64_t)(ao0 + ci * NS + m) * A.ld + g;
            A.X[o] = v;
            A.X[plane + o] = gx;
            A.X[2 * plane + o] = gy;
            A.X[3 * plane + o] = gz;
        }
    }
}

__global__ void ao_eval_d1_kernel(const AoArgs A) {
    __shared__ double etab[64];
    if (threadIdx.x < 64) etab[threadIdx.x] = c_exp2m[threadIdx.x];
    __syncthreads();
    const int sh = blockIdx.y;
    const int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= A.ld) return;
    const int l = A.sh_l[sh];
    if (g >= A.npts) {
        const int n = A.sh_nc[sh] * (2 * l + 1);
        const int64_t plane = (int64_t)A.nao * A.ld;
        for (int i = 0; i < n; ++i)
            for (int c = 0; c < 4; ++c)
                A.X[c * plane + (int64_t)(A.sh_ao0[sh] + i) * A.ld + g] = 0.0;
        return;
    }
    const double dx = A.coords[g * 3] - A.sh_ctr[sh * 3];
    const double dy = A.coords[g * 3 + 1] - A.sh_ctr[sh * 3 + 1];
    const double dz = A.coords[g * 3 + 2] - A.sh_ctr[sh * 3 + 2];
    const double r2 = dx * dx + dy * dy + dz * dz;
    switch (l) {
    case 0: ao_shell_d1<0>(A, sh, g, dx, dy, dz, r2, etab); break;
    case 1: ao_shell_d1<1>(A, sh, g, dx, dy, dz, r2, etab); break;
    case 2: ao_shell_d1<2>(A, sh, g, dx, dy, dz, r2, etab); break;
    default: ao_shell_d1<3>(A, sh, g, dx, dy, dz, r2, etab); break;
    }
}

cudaError_t launch_ao_eval_d1(const AoArgs& a, cudaStream_t s) {
    if (a.ld <= 0 || a.nbas <= 0) return cudaSuccess;
    dim3 grid((unsigned)((a.ld + 127) / 128), (unsigned)a.nbas);
    ao_eval_d1_kernel<<<grid, 128, 0, s>>>(a);
    return cudaGetLastError();
}

cudaError_t launch_ao_eval(const AoArgs& a, cudaStream_t s) {
    if (a.ld <= 0 || a.nbas <= 0) return cudaSuccess;
    dim3 grid((unsigned)((a.ld + 127) / 128), (unsigned)a.nbas);
    ao_eval_kernel<<<grid, 128, 0, s>>>(a);
    return cudaGetLastError();
}

// c2s tables filled by the host (same formula as the host pair builder)
cudaError_t upload_exp_table(const double* t64) {
    return cudaMemcpyToSymbol(c_exp2m, t64, sizeof(double) * 64);
}

cudaError_t upload_c2s_tables(const double* t0, const double* t1,
                              const double* t2, const double* t3) {
    cudaError_t e;
    if ((e = cudaMemcpyToSymbol(c_c2s0, t0, sizeof(double) * 1)) != cudaSuccess) return e;
    if ((e = cudaMemcpyToSymbol(c_c2s1, t1, sizeof(double) * 9)) != cudaSuccess) return e;
    if ((e = cudaMemcpyToSymbol(c_c2s2, t2, sizeof(double) * 30)) != cudaSuccess) return e;
    return cudaMemcpyToSymbol(c_c2s3, t3, sizeof(double) * 70);
}

// -- dense contracted spherical A (validation, gpu/int3c1e.py:230-271) -------
// One thread per (point, pair), run-time L, arrays in local memory.  Uses
// the same pair tables and the same Boys / R / E math as the fused kernels
// but forms the Cartesian block explicitly.
__constant__ float c_c2s_f[4][70];

__device__ void cart_comp(int l, int c, int* i, int* j, int* k) {
    int r = 0;
    while ((r + 1) * (r + 2) / 2 <= c) ++r;
    *i = l - r;
    *j = r - (c - r * (r + 1) / 2);
    *k = l - *i - *j;
}

__device__ int e_index(int la, int lb, int i, int j, int t) {
    // position of (i, j, t) in the packed per-axis list (E^{00}_0 excluded)
    int n = 0;
    for (int ii = 0; ii <= la; ++ii)
        for (int jj = 0; jj <= lb; ++jj)
            for (int tt = 0; tt <= ii + jj; ++tt) {
                if (ii == 0 && jj == 0) continue;
                if (ii == i && jj == j && tt == t) return n;
                ++n;
            }
    return -1;
}

__device__ float e_val(const float* Em, int cnt, int ax, int la, int lb,
                       int i, int j, int t) {
    if (i == 0 && j == 0) return t == 0 ? 1.0f : 0.0f;
    return Em[ax * cnt + e_index(la, lb, i, j, t)];
}

template<int LMAXC>
__device__ void boys_dyn(int L, float T, float* F, const float4* tab) {
    switch (L) {
    case 0: boys_fp32<0>(T, F, tab); break;
    case 1: boys_fp32<1>(T, F, tab); break;
    case 2: boys_fp32<2>(T, F, tab); break;
    case 3: boys_fp32<3>(T, F, tab); break;
    case 4: boys_fp32<4>(T, F, tab); break;
    case 5: boys_fp32<5>(T, F, tab); break;
    default: boys_fp32<6>(T, F, tab); break;
    }
}

struct DenseArgs {
    CosxArgs a;
    int npairs, nao;
    const int* pclass;
    const int* pl;          // (npairs, 2): la, lb
    const int* estride;     // per class, floats
    float* out;             // (npts, nao, nao)
};

__global__ void dense_kernel(const DenseArgs D) {
    const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t total = (int64_t)D.a.npts * D.npairs;
    if (idx >= total) return;
    const int64_t g = idx / D.npairs;
    const int k = (int)(idx - g * D.npairs);
    const CosxArgs& A = D.a;
    const int4 hdr = A.hdr[k];
    const int ia0 = hdr.x, ib0 = hdr.y, pp0 = hdr.z, npp = hdr.w & 0xffff;
    const int cls = D.pclass[k];
    const int la = D.pl[2 * k], lb = D.pl[2 * k + 1], L = la + lb;
    const int nca = (la + 1) * (la + 2) / 2, ncb = (lb + 1) * (lb + 2) / 2;
    int cnt = 0;
    for (int i = 0; i <= la; ++i)
        for (int j = 0; j <= lb; ++j) cnt += i + j + 1;
    cnt -= 1;
    const float gxh = A.gxyz_hi[g], gyh = A.gxyz_hi[A.ld + g], gzh = A.gxyz_hi[2 * A.ld + g];
    const float gxl = A.gxyz_lo[g], gyl = A.gxyz_lo[A.ld + g], gzl = A.gxyz_lo[2 * A.ld + g];
    float Ac[100];
    for (int i = 0; i < 100; ++i) Ac[i] = 0.0f;
    float R[7][7][7];
    for (int m = pp0; m < pp0 + npp; ++m) {
        const float4 ph = A.geo[2 * m], pl = A.geo[2 * m + 1];
        const float dx = (ph.x - gxh) + (pl.x - gxl);
        const float dy = (ph.y - gyh) + (pl.y - gyl);
        const float dz = (ph.z - gzh) + (pl.z - gzl);
        const float r2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
        const float* o = (const float*)(A.om + 5 * (int64_t)m);
        const float T = fmaf(o[0], r2, o[1] * r2);
        float Fb[7];
        boys_dyn<6>(L, T, Fb, A.boys);
        for (int t = 0; t < 7; ++t)
            for (int u = 0; u < 7; ++u)
                for (int v = 0; v < 7; ++v) R[t][u][v] = 0.0f;
        for (int n = L; n >= 0; --n) {
            const int mm = L - n;
            for (int u = 0; u < mm; ++u)
                for (int v = 0; v < mm - u; ++v)
                    for (int t = mm - u - v; t >= 1; --t)
                        R[t][u][v] = (t == 1) ? dx * R[0][u][v]
                            : fmaf(dx, R[t - 1][u][v], (float)(t - 1) * R[t - 2][u][v]);
            for (int v = 0; v < mm; ++v)
                for (int u = mm - v; u >= 1; --u)
                    R[0][u][v] = (u == 1) ? dy * R[0][0][v]
                        : fmaf(dy, R[0][u - 1][v], (float)(u - 1) * R[0][u - 2][v]);
            for (int v = mm; v >= 1; --v)
                R[0][0][v] = (v == 1) ? dz * R[0][0][0]
                    : fmaf(dz, R[0][0][v - 1], (float)(v - 1) * R[0][0][v - 2]);
            R[0][0][0] = fmaf(o[2 + 2 * n], Fb[n], o[3 + 2 * n] * Fb[n]);
        }
        const float* Em = (const float*)A.Ecls[cls] +
                          (int64_t)(m - A.pp_begin[cls]) * D.estride[cls];
        for (int ca = 0; ca < nca; ++ca) {
            int i, j, kk;
            cart_comp(la, ca, &i, &j, &kk);
            for (int cb = 0; cb < ncb; ++cb) {
                int ip, jp, kp;
                cart_comp(lb, cb, &ip, &jp, &kp);
                float s = 0.0f;
                for (int t = 0; t <= i + ip; ++t) {
                    const float ex = e_val(Em, cnt, 0, la, lb, i, ip, t);
                    for (int u = 0; u <= j + jp; ++u) {
                        const float ey = e_val(Em, cnt, 1, la, lb, j, jp, u);
                        for (int v = 0; v <= kk + kp; ++v)
                            s += ex * ey * e_val(Em, cnt, 2, la, lb, kk, kp, v) * R[t][u][v];
                    }
                }
                Ac[ca * ncb + cb] += s;
            }
        }
    }
    const int na = 2 * la + 1, nb = 2 * lb + 1;
    float* row = D.out + g * (int64_t)D.nao * D.nao;
    for (int mu = 0; mu < na; ++mu)
        for (int nu = 0; nu < nb; ++nu) {
            float v = 0.0f;
            for (int ca = 0; ca < nca; ++ca) {
                const float cam = la <= 1 ? (ca == mu ? 1.0f : 0.0f)
                                          : c_c2s_f[la][ca * na + mu];
                if (cam == 0.0f) continue;
                for (int cb = 0; cb < ncb; ++cb) {
                    const float cbn = lb <= 1 ? (cb == nu ? 1.0f : 0.0f)
                                              : c_c2s_f[lb][cb * nb + nu];
                    v += cam * cbn * Ac[ca * ncb + cb];
                }
            }
            row[(int64_t)(ia0 + mu) * D.nao + ib0 + nu] = v;
            row[(int64_t)(ib0 + nu) * D.nao + ia0 + mu] = v;
        }
}

cudaError_t upload_c2s_f(const float* all /* 4 x 70 */) {
    return cudaMemcpyToSymbol(c_c2s_f, all, sizeof(float) * 4 * 70);
}

cudaError_t launch_dense_impl(const CosxArgs& a, int npairs, const int* pclass,
                              const int* pl, const int* estride, int nao,
                              float* out, cudaStream_t s) {
    DenseArgs D;
    D.a = a; D.npairs = npairs; D.nao = nao; D.pclass = pclass; D.pl = pl;
    D.estride = estride; D.out = out;
    const int64_t total = (int64_t)a.npts * npairs;
    if (total <= 0) return cudaSuccess;
    dense_kernel<<<(unsigned)((total + 63) / 64), 64, 0, s>>>(D);
    return cudaGetLastError();
}

// -- Boys batch (tests, gpu/boys.py:181-189) ---------------------------------
template<int L>
__global__ void boys_batch_kernel(const float* __restrict__ t, int64_t n,
                                  const float4* __restrict__ tab,
                                  float* __restrict__ out) {
    __shared__ float4 stab[145 * 5];
    for (int i = threadIdx.x; i < 145 * 5; i += blockDim.x) stab[i] = tab[i];
    __syncthreads();
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float F[L + 1];
    boys_fp32<L>(t[i], F, stab);
#pragma unroll
    for (int m = 0; m <= L; ++m) out[m * n + i] = F[m];
}

cudaError_t launch_boys(const float* t, int64_t n, int nmax,
                        const float4* tab, float* out, cudaStream_t s) {
    if (n <= 0) return cudaSuccess;
    const unsigned blocks = (unsigned)((n + 255) / 256);
    switch (nmax) {
    case 0: boys_batch_kernel<0><<<blocks, 256, 0, s>>>(t, n, tab, out); break;
    case 1: boys_batch_kernel<1><<<blocks, 256, 0, s>>>(t, n, tab, out); break;
    case 2: boys_batch_kernel<2><<<blocks, 256, 0, s>>>(t, n, tab, out); break;
    case 3: boys_batch_kernel<3><<<blocks, 256, 0, s>>>(t, n, tab, out); break;
    case 4: boys_batch_kernel<4><<<blocks, 256, 0, s>>>(t, n, tab, out); break;
    case 5: boys_batch_kernel<5><<<blocks, 256, 0, s>>>(t, n, tab, out); break;
    case 6: boys_batch_kernel<6><<<blocks, 256, 0, s>>>(t, n, tab, out); break;
    default: return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}

}  // namespace wb

namespace wb {

// -- FP32 FMA throughput probe (the roofline denominator of the FP32-pipe
// kernels): 8 independent FMA chains per thread, nothing but FFMA in the
// loop; each thread writes one value so nothing is optimised away.
__global__ void fma_probe_kernel(int64_t iters, float* __restrict__ out) {
    float a0 = threadIdx.x * 1e-7f, a1 = a0 + 1e-7f, a2 = a0 + 2e-7f,
          a3 = a0 + 3e-7f, a4 = a0 + 4e-7f, a5 = a0 + 5e-7f, a6 = a0 + 6e-7f,
          a7 = a0 + 7e-7f;
    const float m = 0.999999f, c = 1e-7f;
    for (int64_t i = 0; i < iters; ++i) {
#pragma unroll
        for (int k = 0; k < 16; ++k) {
            a0 = fmaf(a0, m, c); a1 = fmaf(a1, m, c); a2 = fmaf(a2, m, c);
            a3 = fmaf(a3, m, c); a4 = fmaf(a4, m, c); a5 = fmaf(a5, m, c);
            a6 = fmaf(a6, m, c); a7 = fmaf(a7, m, c);
        }
    }
    out[(int64_t)blockIdx.x * blockDim.x + threadIdx.x] =
        a0 + a1 + a2 + a3 + a4 + a5 + a6 + a7;
}

// the same with packed FMAs (fma.rn.f32x2: two FP32 FMAs per instruction)
__global__ void fma2_probe_kernel(int64_t iters, float* __restrict__ out) {
    unsigned long long a[8];
    const float b0 = threadIdx.x * 1e-7f;
    for (int k = 0; k < 8; ++k) {
        const float lo = b0 + 2 * k * 1e-7f, hi = lo + 1e-7f;
        asm("mov.b64 %0, {%1, %2};" : "=l"(a[k]) : "f"(lo), "f"(hi));
    }
    unsigned long long m, c;
    asm("mov.b64 %0, {%1, %1};" : "=l"(m) : "f"(0.999999f));
    asm("mov.b64 %0, {%1, %1};" : "=l"(c) : "f"(1e-7f));
    for (int64_t i = 0; i < iters; ++i) {
#pragma unroll
        for (int k = 0; k < 16; ++k) {
#pragma unroll
            for (int r = 0; r < 8; ++r)
                asm volatile("fma.rn.f32x2 %0, %0, %1, %2;" : "+l"(a[r]) : "l"(m), "l"(c));
        }
    }
    float s = 0.0f;
    for (int k = 0; k < 8; ++k) {
        float lo, hi;
        asm("mov.b64 {%0, %1}, %2;" : "=f"(lo), "=f"(hi) : "l"(a[k]));
        s += lo + hi;
    }
    out[(int64_t)blockIdx.x * blockDim.x + threadIdx.x] = s;
}

cudaError_t launch_fma_probe(int64_t iters, int blocks, int threads,
                             float* out, cudaStream_t s, bool packed) {
    if (packed)
        fma2_probe_kernel<<<blocks, threads, 0, s>>>(iters, out);
    else
        fma_probe_kernel<<<blocks, threads, 0, s>>>(iters, out);
    return cudaGetLastError();
}

// -- screen mask (test aid) ---------------------------------------------------
// keep[blk * npairs + k] = 1 where the fused G kernels keep task (blk, k)
// at block level lv (blocks of 32 << lv points): the same screen_pair call,
// on the same block statistics and pair data, as the class kernels make.
__global__ void screen_mask_kernel(const CosxArgs A, const int lv, const int npairs,
                                   unsigned char* __restrict__ keep) {
    const int64_t total = (int64_t)A.nblk[lv] * npairs;
    for (int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; idx < total;
         idx += (int64_t)gridDim.x * blockDim.x) {
        const int blk = (int)(idx / npairs);
        const int k = (int)(idx - (int64_t)blk * npairs);
        int c = 0;
        while (c < kClasses - 1 && !(k >= A.cls_pb[c] && k < A.cls_pe[c])) ++c;
        bool kp = true;
        if (A.tol > 0.0f) {
            const int2 sh = A.pshell[k];
            const float* ms = A.blk_msh[lv] + (int64_t)blk * A.nvshell;
            kp = screen_pair(A.tol, A.bnd + A.pp_begin[c], A.bpref + A.pp_begin[c],
                             A.blk_cr[lv][blk], A.khdr[k], A.ptau[k],
                             fmaxf(ms[sh.x], ms[sh.y]));
        }
        keep[idx] = kp ? 1 : 0;
    }
}

cudaError_t launch_screen_mask(const CosxArgs& a, int lv, int npairs,
                               unsigned char* keep, cudaStream_t s) {
    const int64_t total = (int64_t)a.nblk[lv] * npairs;
    if (total <= 0) return cudaSuccess;
    screen_mask_kernel<<<(unsigned)grid_stride_blocks(total, 256, 16), 256, 0, s>>>(
        a, lv, npairs, keep);
    return cudaGetLastError();
}

}  // namespace wb
