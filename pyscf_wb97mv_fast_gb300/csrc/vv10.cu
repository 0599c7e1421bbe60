// VV10 non-local correlation double sum (reference: gpu/vv10.py:47-98,
// :128-164, :167-240; formula of libdft VXC_vv10nlc).
//
//   g_ij = R^2 w0_i + k_i,  gp_ij = R^2 w0_j + k_j,  gt = g + gp
//   T  = q_j / (g gp gt),   Tu = T (1/g + 1/gt),   Tw = Tu R^2
//   F_i = -1.5 sum_j T,  U_i = sum_j Tu,  W_i = sum_j Tw
//
// One thread per outer point, inner points staged through shared memory in
// 256-point tiles.  Inside a tile the sums run in FP32 over 16 pairs at a
// time, and those partials join Kahan-compensated tile sums; across tiles
// they accumulate in FP64 in a fixed order: no atomics, bitwise
// reproducible.  One reciprocal per pair (rcp.approx plus one Newton step):
// T = q / (g gp gt), Tu = T (g + gt) gp / (g gp gt).
//
// Distance pruning on the device: per 256-point tile the centroid, radius,
// sum q, min w0 and min kappa (FP64); a (block, tile) pair is skipped when
// the reference's bounds (gpu/vv10.py:21-31)
//   F <= sum_J q / (g gp (g + gp)),  U <= 2 F / g_min,  W <= U Rmax^2
// with g, gp at the minimum distance are all below tile_tol; tile_tol = 0
// keeps every pair.
#include <cmath>

#include "launch.hpp"

namespace wb {

constexpr int kVvTile = 256;

// one Newton step on the approximate reciprocal (1 = on)
#ifndef WB_VV10_NEWTON
#define WB_VV10_NEWTON 1
#endif

struct VvTileStats {
    double cx, cy, cz, rad, qsum, w0min, kmin, pad;
};

size_t vv10_workspace_bytes(int64_t n) {
    const int64_t nt = (n + kVvTile - 1) / kVvTile;
    return (size_t)nt * sizeof(VvTileStats) + 256;
}

__global__ void vv10_tile_stats_kernel(const float* __restrict__ xyz,
                                       const float* __restrict__ q,
                                       const float* __restrict__ w0,
                                       const float* __restrict__ kap,
                                       int64_t n, VvTileStats* __restrict__ st) {
    // one warp per tile
    const int64_t tile = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    const int64_t nt = (n + kVvTile - 1) / kVvTile;
    if (tile >= nt) return;
    const int64_t i0 = tile * kVvTile;
    const int64_t i1 = min(n, i0 + kVvTile);
    double sx = 0, sy = 0, sz = 0, sq = 0, mw = INFINITY, mk = INFINITY;
    for (int64_t i = i0 + lane; i < i1; i += 32) {
        sx += xyz[3 * i]; sy += xyz[3 * i + 1]; sz += xyz[3 * i + 2];
        sq += q[i];
        mw = fmin(mw, (double)w0[i]);
        mk = fmin(mk, (double)kap[i]);
    }
    for (int o = 16; o > 0; o >>= 1) {
        sx += __shfl_xor_sync(0xffffffffu, sx, o);
        sy += __shfl_xor_sync(0xffffffffu, sy, o);
        sz += __shfl_xor_sync(0xffffffffu, sz, o);
        sq += __shfl_xor_sync(0xffffffffu, sq, o);
        mw = fmin(mw, __shfl_xor_sync(0xffffffffu, mw, o));
        mk = fmin(mk, __shfl_xor_sync(0xffffffffu, mk, o));
    }
    const double cnt = (double)(i1 - i0);
    const double cx = sx / cnt, cy = sy / cnt, cz = sz / cnt;
    double r = 0.0;
    for (int64_t i = i0 + lane; i < i1; i += 32) {
        const double dx = xyz[3 * i] - cx, dy = xyz[3 * i + 1] - cy,
                     dz = xyz[3 * i + 2] - cz;
        r = fmax(r, sqrt(dx * dx + dy * dy + dz * dz));
    }
    for (int o = 16; o > 0; o >>= 1) r = fmax(r, __shfl_xor_sync(0xffffffffu, r, o));
    if (lane == 0) {
        VvTileStats s;
        s.cx = cx; s.cy = cy; s.cz = cz; s.rad = r * (1.0 + 1e-12) + 1e-12;
        s.qsum = sq; s.w0min = mw; s.kmin = mk; s.pad = 0.0;
        st[tile] = s;
    }
}

__device__ __forceinline__ bool vv10_keep(const VvTileStats& a,
                                          const VvTileStats& b, double tol) {
    if (tol <= 0.0) return true;
    const double dx = a.cx - b.cx, dy = a.cy - b.cy, dz = a.cz - b.cz;
    const double dist = sqrt(dx * dx + dy * dy + dz * dz);
    const double rmin = fmax(dist - a.rad - b.rad, 0.0);
    const double rmax = dist + a.rad + b.rad;
    const double gmin = rmin * rmin * a.w0min + a.kmin;
    const double gpmin = rmin * rmin * b.w0min + b.kmin;
    const double bf = b.qsum / (gmin * gpmin * (gmin + gpmin));
    const double bu = bf * 2.0 / gmin;
    const double bw = bu * rmax * rmax;
    return fmax(fmax(bf, bu), bw) >= tol;
}

// One outer point: its coordinates, w0 and kappa.
struct VvOuter { float x, y, z, w0, k; };

// FP64 running sums of one outer point and its count of pairs computed.
struct VvSums {
    double f = 0.0, u = 0.0, w = 0.0;
    unsigned long long pairs = 0;
};

// Index i must be valid; callers clamp it for threads past the end.
__device__ __forceinline__ VvOuter vv_load_outer(const float* __restrict__ xyz,
                                                 const float* __restrict__ w0,
                                                 const float* __restrict__ kap,
                                                 const int64_t i) {
    return VvOuter{xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2], w0[i], kap[i]};
}

// F carries the -3/2 of the VV10 kernel; U and W are the plain sums.
__device__ __forceinline__ void vv_store(const VvSums& acc, const int64_t i,
                                         double* __restrict__ F,
                                         double* __restrict__ U,
                                         double* __restrict__ W) {
    F[i] = acc.f * -1.5;
    U[i] = acc.u;
    W[i] = acc.w;
}

// Inner point j into shared slot t: (x, y, z, q) and (w0, kappa).
__device__ __forceinline__ void vv_stage(float4* sp, float2* sk, const int t,
                                         const float* __restrict__ xyz,
                                         const float* __restrict__ q,
                                         const float* __restrict__ w0,
                                         const float* __restrict__ kap,
                                         const int64_t j) {
    const float* c = xyz + 3 * j;
    sp[t] = make_float4(c[0], c[1], c[2], q[j]);
    sk[t] = make_float2(w0[j], kap[j]);
}

// Compensated accumulation of x into (sum, comp) (Kahan, 1965).
__device__ __forceinline__ void kahan_add(float& sum, float& comp, const float x) {
    const float xc = x - comp;
    const float t = sum + xc;
    comp = (t - sum) - xc;
    sum = t;
}

// Block-wide integer total of v, added once per block to *total (the
// order of an integer sum does not matter).  Every thread of the block
// must call it.
template<int NT>
__device__ __forceinline__ void vv_block_count(unsigned long long v,
                                               unsigned long long* total) {
    __shared__ unsigned long long warp_part[NT / 32];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if ((threadIdx.x & 31) == 0) warp_part[threadIdx.x >> 5] = v;
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned long long t = 0;
#pragma unroll
        for (int w = 0; w < NT / 32; ++w) t += warp_part[w];
        atomicAdd(total, t);
    }
}

// The pairs of one outer point with one staged inner tile (m points), the
// one-reciprocal form: inv = 1/(g gp gt) from rcp.approx and one Newton
// step, T = q inv and, with 1/g + 1/gt = (g + gt) gp inv, Tu = T (g + gt)
// gp inv.  Plain FP32 sums over 16 pairs, merged into Kahan-compensated
// tile sums once per 16 pairs; the tile sums join the FP64 totals.  Shared
// by the single-molecule and the batched kernels (same arithmetic, same
// order).
__device__ __forceinline__ void vv10_tile_fast(const VvOuter& o, const float4* sp,
                                               const float2* sk, const int m,
                                               VvSums& acc) {
    float fs = 0.f, fc = 0.f, us = 0.f, uc = 0.f, ws = 0.f, wc = 0.f;
    auto pair = [&](const int t, float& pf, float& pu, float& pw) {
        const float4 pj = sp[t];
        const float2 kj = sk[t];
        const float dx = o.x - pj.x, dy = o.y - pj.y, dz = o.z - pj.z;
        const float r2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
        const float g = fmaf(r2, o.w0, o.k);
        const float gp = fmaf(r2, kj.x, kj.y);
        const float gt = g + gp;
        const float pr = g * gp * gt;
        float inv;
        asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(inv) : "f"(pr));
        if (WB_VV10_NEWTON) inv = fmaf(inv, fmaf(-pr, inv, 1.0f), inv);
        const float T = pj.w * inv;
        const float Tu = T * ((g + gt) * gp * inv);
        pf += T;
        pu += Tu;
        pw = fmaf(Tu, r2, pw);
    };
    for (int t0 = 0; t0 < m; t0 += 16) {
        float pf = 0.f, pu = 0.f, pw = 0.f;
        if (t0 + 16 <= m) {
#pragma unroll
            for (int t = 0; t < 16; ++t) pair(t0 + t, pf, pu, pw);
        } else {
            for (int t = t0; t < m; ++t) pair(t, pf, pu, pw);
        }
        kahan_add(fs, fc, pf);
        kahan_add(us, uc, pu);
        kahan_add(ws, wc, pw);
    }
    acc.f += (double)fs;
    acc.u += (double)us;
    acc.w += (double)ws;
    acc.pairs += (unsigned long long)m;
}

// Warp 0 of a block: the keep decisions of the 32 inner tiles
// [u0, u0 + 32) against outer tile `self` (tiles at or past u_end are
// dropped), one per lane, as one ballot word in keep_word.  A decision is
// an FP64 bound with a square root and two divisions; evaluating 32 at
// once keeps that latency off the block's per-tile path (one thread
// evaluating each tile in turn while the block waited cost 12 % of the
// sum at tile_tol 1e-12).
__device__ __forceinline__ void vv_keep_word(const VvTileStats* __restrict__ st,
                                             const int64_t self, const int64_t u0,
                                             const int64_t u_end, const double tol,
                                             unsigned* keep_word) {
    const int64_t u = u0 + threadIdx.x;
    const bool kp = u < u_end && vv10_keep(st[self], st[u], tol);
    const unsigned bits = __ballot_sync(0xffffffffu, kp);
    if (threadIdx.x == 0) *keep_word = bits;
}

// One block per 256-point outer tile.  Warp 0 decides, 32 inner tiles at
// a time, which of them the block needs (the decision words sit in a
// two-slot parity buffer, so the next word cannot overwrite one still
// being read); the block stages each kept tile and every live thread runs
// its pairs.
__global__ void __launch_bounds__(kVvTile, 5)
vv10_sum_kernel(const float* __restrict__ xyz, const float* __restrict__ q,
                const float* __restrict__ w0, const float* __restrict__ kap,
                int64_t n, double tol, const VvTileStats* __restrict__ st,
                double* __restrict__ F, double* __restrict__ U,
                double* __restrict__ W, unsigned long long* __restrict__ kept) {
    __shared__ float4 sp[kVvTile];      // x, y, z, q
    __shared__ float2 sk[kVvTile];      // w0, kappa
    __shared__ unsigned s_keep[2];
    const int64_t i = (int64_t)blockIdx.x * kVvTile + threadIdx.x;
    const bool live = i < n;
    const VvOuter o = vv_load_outer(xyz, w0, kap, live ? i : n - 1);
    const int64_t ntiles = (n + kVvTile - 1) / kVvTile;
    VvSums acc;
    for (int64_t jt = 0; jt < ntiles; ++jt) {
        const int sl = (int)((jt >> 5) & 1);
        if ((jt & 31) == 0 && threadIdx.x < 32)
            vv_keep_word(st, blockIdx.x, jt, ntiles, tol, &s_keep[sl]);
        const int64_t j = jt * kVvTile + threadIdx.x;
        __syncthreads();
        if (!((s_keep[sl] >> (jt & 31)) & 1u)) continue;  // uniform across the block
        if (j < n) vv_stage(sp, sk, threadIdx.x, xyz, q, w0, kap, j);
        __syncthreads();
        if (live)
            vv10_tile_fast(o, sp, sk, (int)min((int64_t)kVvTile, n - jt * kVvTile),
                           acc);
        __syncthreads();
    }
    if (live) vv_store(acc, i, F, U, W);
    if (kept) vv_block_count<kVvTile>(acc.pairs, kept);
}

// Packed form (-DWB_VV10_PACKED=1; the default is the kernel above): two
// outer points per thread, i and i + 256 of a 512-point block, carried
// as the two halves of f32x2 registers, so that each packed instruction
// (add / mul / fma .f32x2, sm_100+) does one step of two pairs.  The inner
// tile is staged duplicated ({x, x, y, y}, {z, z, q, q}, {w0, w0, k, k}), so
// every inner value is already a packed operand.  Per pair the same
// operations as the one-reciprocal form above, in the same order (two
// rcp.approx + one packed Newton step), 16-pair partial sums merged into
// Kahan-compensated tile sums, FP64 across tiles: no atomics, bitwise
// reproducible.  An outer block keeps an inner tile if either of its two
// 256-point tiles does.  Measured on the bench's VV10 grid (209,707 points)
// it took 36.8 ms against 36.4 ms for the scalar kernel: the double sum is
// bound by the FP32 pipe itself (73 % of its cycles), not by instruction
// issue, and a packed FMA occupies the pipe for both halves (the packed
// probe, wb_fp32x2_fma_probe, reaches 80.5 TFLOP/s against 76.8 for scalar
// FMAs: the issue slots it frees do not add FP32 throughput).
#ifndef WB_VV10_PACKED
#define WB_VV10_PACKED 0
#endif

namespace {

typedef unsigned long long f2r;     // two f32 in one 64-bit register

__device__ __forceinline__ f2r pk(const float lo, const float hi) {
    f2r r;
    asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(lo), "f"(hi));
    return r;
}
__device__ __forceinline__ void upk(const f2r r, float& lo, float& hi) {
    asm("mov.b64 {%0, %1}, %2;" : "=f"(lo), "=f"(hi) : "l"(r));
}
__device__ __forceinline__ f2r add2(const f2r a, const f2r b) {
    f2r d;
    asm("add.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
    return d;
}
__device__ __forceinline__ f2r sub2(const f2r a, const f2r b) {
    f2r d;
    asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
    return d;
}
__device__ __forceinline__ f2r mul2(const f2r a, const f2r b) {
    f2r d;
    asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
    return d;
}
__device__ __forceinline__ f2r fma2(const f2r a, const f2r b, const f2r c) {
    f2r d;
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(d) : "l"(a), "l"(b), "l"(c));
    return d;
}
// sign flip of both halves (an integer op, off the FP32 pipe)
__device__ __forceinline__ f2r neg2(const f2r a) { return a ^ 0x8000000080000000ull; }
__device__ __forceinline__ f2r rcp2(const f2r a) {
    float lo, hi;
    upk(a, lo, hi);
    asm("rcp.approx.ftz.f32 %0, %0;" : "+f"(lo));
    asm("rcp.approx.ftz.f32 %0, %0;" : "+f"(hi));
    return pk(lo, hi);
}

constexpr int kVvOuter = 2 * kVvTile;

__global__ void __launch_bounds__(kVvTile)
vv10_sum_packed_kernel(const float* __restrict__ xyz, const float* __restrict__ q,
                       const float* __restrict__ w0, const float* __restrict__ kap,
                       int64_t n, double tol, const VvTileStats* __restrict__ st,
                       double* __restrict__ F, double* __restrict__ U,
                       double* __restrict__ W, unsigned long long* __restrict__ kept) {
    __shared__ float4 sxy[kVvTile];     // x, x, y, y
    __shared__ float4 szq[kVvTile];     // z, z, q, q
    __shared__ float4 swk[kVvTile];     // w0, w0, kappa, kappa
    __shared__ int s_keep[2];
    const int64_t i0 = (int64_t)blockIdx.x * kVvOuter + threadIdx.x;
    const int64_t i1 = i0 + kVvTile;
    const bool a0 = i0 < n, a1 = i1 < n;
    const VvOuter o0 = vv_load_outer(xyz, w0, kap, a0 ? i0 : n - 1);
    const VvOuter o1 = vv_load_outer(xyz, w0, kap, a1 ? i1 : n - 1);
    const f2r xi = pk(o0.x, o1.x), yi = pk(o0.y, o1.y), zi = pk(o0.z, o1.z);
    const f2r w0i = pk(o0.w0, o1.w0), ki = pk(o0.k, o1.k);
    const f2r one = pk(1.0f, 1.0f);
    const int64_t nt = (n + kVvTile - 1) / kVvTile;
    const int64_t ob = 2 * (int64_t)blockIdx.x;           // outer stats tiles
    double f64[2] = {0.0, 0.0}, u64[2] = {0.0, 0.0}, w64[2] = {0.0, 0.0};
    unsigned long long nkept = 0;
    for (int64_t jt = 0; jt < nt; ++jt) {
        if (threadIdx.x == 0) {
            int kp = vv10_keep(st[ob], st[jt], tol);
            if (ob + 1 < nt) kp = kp || vv10_keep(st[ob + 1], st[jt], tol);
            s_keep[jt & 1] = kp;
        }
        const int64_t j = jt * kVvTile + threadIdx.x;
        __syncthreads();
        if (!s_keep[jt & 1]) continue;  // uniform across the block
        if (j < n) {
            const float xj = xyz[3 * j], yj = xyz[3 * j + 1], zj = xyz[3 * j + 2];
            const float qj = q[j], wj = w0[j], kj = kap[j];
            sxy[threadIdx.x] = make_float4(xj, xj, yj, yj);
            szq[threadIdx.x] = make_float4(zj, zj, qj, qj);
            swk[threadIdx.x] = make_float4(wj, wj, kj, kj);
        }
        __syncthreads();
        const int m = (int)min((int64_t)kVvTile, n - jt * kVvTile);
        f2r fs = 0, fc = 0, us = 0, uc = 0, ws = 0, wc = 0;
        auto kahan_add2 = [](f2r& sum, f2r& comp, const f2r x) {
            const f2r xc = sub2(x, comp);
            const f2r t = add2(sum, xc);
            comp = sub2(sub2(t, sum), xc);
            sum = t;
        };
        auto pair = [&](const int t, f2r& pf, f2r& pu, f2r& pw) {
            const float4 a = sxy[t], b = szq[t], c = swk[t];
            const f2r xj = pk(a.x, a.y), yj = pk(a.z, a.w);
            const f2r zj = pk(b.x, b.y), qj = pk(b.z, b.w);
            const f2r wj = pk(c.x, c.y), kj = pk(c.z, c.w);
            const f2r dx = sub2(xi, xj), dy = sub2(yi, yj), dz = sub2(zi, zj);
            const f2r r2 = fma2(dx, dx, fma2(dy, dy, mul2(dz, dz)));
            const f2r g = fma2(r2, w0i, ki);
            const f2r gp = fma2(r2, wj, kj);
            const f2r gt = add2(g, gp);
            const f2r pr = mul2(mul2(g, gp), gt);
            f2r inv = rcp2(pr);
            if (WB_VV10_NEWTON) inv = fma2(inv, fma2(neg2(pr), inv, one), inv);
            const f2r T = mul2(qj, inv);
            const f2r Tu = mul2(T, mul2(mul2(add2(g, gt), gp), inv));
            pf = add2(pf, T);
            pu = add2(pu, Tu);
            pw = fma2(Tu, r2, pw);
        };
        for (int t0 = 0; t0 < m; t0 += 16) {
            f2r pf = 0, pu = 0, pw = 0;
            if (t0 + 16 <= m) {
#pragma unroll
                for (int t = 0; t < 16; ++t) pair(t0 + t, pf, pu, pw);
            } else {
                for (int t = t0; t < m; ++t) pair(t, pf, pu, pw);
            }
            kahan_add2(fs, fc, pf);
            kahan_add2(us, uc, pu);
            kahan_add2(ws, wc, pw);
        }
        float lo, hi;
        upk(fs, lo, hi); f64[0] += (double)lo; f64[1] += (double)hi;
        upk(us, lo, hi); u64[0] += (double)lo; u64[1] += (double)hi;
        upk(ws, lo, hi); w64[0] += (double)lo; w64[1] += (double)hi;
        nkept += (unsigned long long)m * ((a0 ? 1 : 0) + (a1 ? 1 : 0));
        __syncthreads();
    }
    VvSums s0, s1;
    s0.f = f64[0]; s0.u = u64[0]; s0.w = w64[0];
    s1.f = f64[1]; s1.u = u64[1]; s1.w = w64[1];
    if (a0) vv_store(s0, i0, F, U, W);
    if (a1) vv_store(s1, i1, F, U, W);
    if (kept) vv_block_count<kVvTile>(nkept, kept);
}

}  // namespace

// -- batched form: several molecules' point sets in one launch -------------
// The points of molecule m are [off_m, off_m+1) of the concatenated arrays
// and are cut into 256-point tiles that never straddle two molecules:
// tile t covers [tstart[t], tstart[t] + tlen[t]) of molecule tmol[t], and
// molecule m owns tiles mtile[m] .. mtile[m + 1] - 1.  One block per outer
// tile; its inner tiles are those of its own molecule, in order, so every
// molecule's sums are bitwise those of its single-molecule call.

__global__ void vv10_tile_stats_seg_kernel(const float* __restrict__ xyz,
                                           const float* __restrict__ q,
                                           const float* __restrict__ w0,
                                           const float* __restrict__ kap,
                                           const VvSeg sg, VvTileStats* __restrict__ st) {
    const int64_t tile = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (tile >= sg.ntiles) return;
    const int64_t i0 = sg.tstart[tile];
    const int64_t i1 = i0 + sg.tlen[tile];
    double sx = 0, sy = 0, sz = 0, sq = 0, mw = INFINITY, mk = INFINITY;
    for (int64_t i = i0 + lane; i < i1; i += 32) {
        sx += xyz[3 * i]; sy += xyz[3 * i + 1]; sz += xyz[3 * i + 2];
        sq += q[i];
        mw = fmin(mw, (double)w0[i]);
        mk = fmin(mk, (double)kap[i]);
    }
    for (int o = 16; o > 0; o >>= 1) {
        sx += __shfl_xor_sync(0xffffffffu, sx, o);
        sy += __shfl_xor_sync(0xffffffffu, sy, o);
        sz += __shfl_xor_sync(0xffffffffu, sz, o);
        sq += __shfl_xor_sync(0xffffffffu, sq, o);
        mw = fmin(mw, __shfl_xor_sync(0xffffffffu, mw, o));
        mk = fmin(mk, __shfl_xor_sync(0xffffffffu, mk, o));
    }
    const double cnt = (double)(i1 - i0);
    const double cx = sx / cnt, cy = sy / cnt, cz = sz / cnt;
    double r = 0.0;
    for (int64_t i = i0 + lane; i < i1; i += 32) {
        const double dx = xyz[3 * i] - cx, dy = xyz[3 * i + 1] - cy,
                     dz = xyz[3 * i + 2] - cz;
        r = fmax(r, sqrt(dx * dx + dy * dy + dz * dz));
    }
    for (int o = 16; o > 0; o >>= 1) r = fmax(r, __shfl_xor_sync(0xffffffffu, r, o));
    if (lane == 0) {
        VvTileStats s;
        s.cx = cx; s.cy = cy; s.cz = cz; s.rad = r * (1.0 + 1e-12) + 1e-12;
        s.qsum = sq; s.w0min = mw; s.kmin = mk; s.pad = 0.0;
        st[tile] = s;
    }
}

__global__ void __launch_bounds__(kVvTile)
vv10_sum_seg_kernel(const float* __restrict__ xyz, const float* __restrict__ q,
                    const float* __restrict__ w0, const float* __restrict__ kap,
                    const VvSeg sg, double tol, const VvTileStats* __restrict__ st,
                    double* __restrict__ F, double* __restrict__ U,
                    double* __restrict__ W, unsigned long long* __restrict__ kept) {
    __shared__ float4 sp[kVvTile];      // x, y, z, q
    __shared__ float2 sk[kVvTile];      // w0, kappa
    __shared__ unsigned s_keep[2];
    const int64_t t = blockIdx.x;
    const int mol = sg.tmol[t];
    const int64_t i = sg.tstart[t] + threadIdx.x;
    const bool live = (int)threadIdx.x < sg.tlen[t];
    const VvOuter o = vv_load_outer(xyz, w0, kap, live ? i : sg.tstart[t]);
    VvSums acc;
    const int jt0 = sg.mtile[mol], jt1 = sg.mtile[mol + 1];
    for (int jt = jt0; jt < jt1; ++jt) {
        const int k = jt - jt0;          // the tile's index within its molecule
        const int sl = (k >> 5) & 1;
        if ((k & 31) == 0 && threadIdx.x < 32)
            vv_keep_word(st, t, jt, jt1, tol, &s_keep[sl]);
        const int m = sg.tlen[jt];
        const int64_t j = sg.tstart[jt] + threadIdx.x;
        __syncthreads();
        if (!((s_keep[sl] >> (k & 31)) & 1u)) continue;  // uniform across the block
        if ((int)threadIdx.x < m) vv_stage(sp, sk, threadIdx.x, xyz, q, w0, kap, j);
        __syncthreads();
        if (live) vv10_tile_fast(o, sp, sk, m, acc);
        __syncthreads();
    }
    if (live) vv_store(acc, i, F, U, W);
    if (kept) vv_block_count<kVvTile>(acc.pairs, kept);
}

cudaError_t launch_vv10_seg(const float* xyz, const float* q, const float* w0,
                            const float* kap, const VvSeg& sg, double tile_tol,
                            double* F, double* U, double* W, void* stats,
                            unsigned long long* kept, cudaStream_t s) {
    if (sg.ntiles <= 0) return cudaSuccess;
    VvTileStats* st = static_cast<VvTileStats*>(stats);
    vv10_tile_stats_seg_kernel<<<(unsigned)((sg.ntiles * 32 + 127) / 128), 128, 0, s>>>(
        xyz, q, w0, kap, sg, st);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    vv10_sum_seg_kernel<<<(unsigned)sg.ntiles, kVvTile, 0, s>>>(xyz, q, w0, kap, sg,
                                                               tile_tol, st, F, U, W,
                                                               kept);
    return cudaGetLastError();
}

size_t vv10_tile_stats_bytes(int64_t ntiles) {
    return (size_t)ntiles * sizeof(VvTileStats);
}

cudaError_t launch_vv10(const float* xyz, const float* q, const float* w0,
                        const float* kap, int64_t n, double tile_tol,
                        double* F, double* U, double* W, void* ws,
                        cudaStream_t s) {
    if (n <= 0) return cudaSuccess;
    const int64_t nt = (n + kVvTile - 1) / kVvTile;
    char* base = (char*)ws;
    unsigned long long* kept = (unsigned long long*)base;
    VvTileStats* st = (VvTileStats*)(base + 256);
    cudaError_t e = cudaMemsetAsync(kept, 0, sizeof(unsigned long long), s);
    if (e != cudaSuccess) return e;
    vv10_tile_stats_kernel<<<(unsigned)((nt * 32 + 127) / 128), 128, 0, s>>>(
        xyz, q, w0, kap, n, st);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    if (WB_VV10_PACKED) {
        const int64_t nb = (n + kVvOuter - 1) / kVvOuter;
        vv10_sum_packed_kernel<<<(unsigned)nb, kVvTile, 0, s>>>(
            xyz, q, w0, kap, n, tile_tol, st, F, U, W, kept);
    } else {
        vv10_sum_kernel<<<(unsigned)nt, kVvTile, 0, s>>>(xyz, q, w0, kap, n,
                                                         tile_tol, st, F, U, W,
                                                         kept);
    }
    return cudaGetLastError();
}

}  // namespace wb

// ---------------------------------------------------------------------------
// Allocation-free variant of wb_vv10_kernel_sum.
//
// Some callers of this library cannot let it allocate device memory: a
// host framework that reserves all of the GPU memory up front and hands
// out fixed arenas (a cudaMalloc in the middle of a request would fail or
// stall the device), or a caller that must keep every CUDA call of the
// hot loop free of the allocator.  For them the VV10 tile statistics and
// the kept-pair counter live in this file-scope device array instead of a
// cudaMallocAsync'd workspace.  Its size is fixed at build time, so the
// entry point serves at most WB_VV10_NOALLOC_MAX_POINTS points, and every
// GPU that loads the library holds it until the process exits.
// ---------------------------------------------------------------------------
#include <string>

#include "wb97mv_gb300.h"

namespace wb {
// the calling thread's wb_last_error() message (defined with the C ABI)
void set_last_error(const std::string& msg);
}

namespace {

constexpr int64_t kNoallocMaxTiles =
    (WB_VV10_NOALLOC_MAX_POINTS + wb::kVvTile - 1) / wb::kVvTile;
constexpr size_t kNoallocBytes =
    256 + sizeof(wb::VvTileStats) * (size_t)kNoallocMaxTiles;

// [0, 256): kept-pair counter; [256, ...): one VvTileStats per tile
static __device__ __align__(256) unsigned char g_vv10_scratch[kNoallocBytes];

int noalloc_fail(int code, const char* msg, cudaError_t e = cudaSuccess) {
    std::string m(msg);
    if (e != cudaSuccess) m += std::string(": ") + cudaGetErrorString(e);
    wb::set_last_error(m);
    return code;
}

}  // namespace

extern "C" int wb_vv10_kernel_sum_noalloc(const float* xyz, const float* q,
                                          const float* w0, const float* kappa,
                                          int64_t n, double tile_tol,
                                          double* f_out, double* u_out,
                                          double* w_out, void* stream,
                                          int64_t* pairs_kept) {
    if (n < 0 || !(tile_tol >= 0.0))
        return noalloc_fail(WB_ERR_INVALID_ARGUMENT,
                            "wb_vv10_kernel_sum_noalloc: n must be >= 0 and "
                            "tile_tol >= 0");
    if (n > WB_VV10_NOALLOC_MAX_POINTS)
        return noalloc_fail(WB_ERR_INVALID_ARGUMENT,
                            "wb_vv10_kernel_sum_noalloc: n exceeds "
                            "WB_VV10_NOALLOC_MAX_POINTS (the size of its "
                            "static scratch); use wb_vv10_kernel_sum");
    if (n && (!xyz || !q || !w0 || !kappa || !f_out || !u_out || !w_out))
        return noalloc_fail(WB_ERR_INVALID_ARGUMENT,
                            "wb_vv10_kernel_sum_noalloc: null pointer");
    if (n == 0) {
        if (pairs_kept) *pairs_kept = 0;
        return WB_OK;
    }
    // the array's device address in the current context, looked up on every
    // call (a host-side table query, no allocation), so that a context torn
    // down and made again never leaves a stale address behind
    void* scratch = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&scratch, g_vv10_scratch);
    if (e != cudaSuccess || !scratch)
        return noalloc_fail(WB_ERR_CUDA,
                            "wb_vv10_kernel_sum_noalloc: cudaGetSymbolAddress", e);
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    // launch_vv10 zeroes the counter and overwrites every tile record it
    // reads; nothing else in the array must start at zero
    e = wb::launch_vv10(xyz, q, w0, kappa, n, tile_tol, f_out, u_out, w_out,
                        scratch, s);
    if (e != cudaSuccess)
        return noalloc_fail(WB_ERR_CUDA, "wb_vv10_kernel_sum_noalloc: launch", e);
    if (pairs_kept) {
        unsigned long long kept = 0;
        e = cudaMemcpyAsync(&kept, scratch, sizeof(kept), cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s);
        if (e != cudaSuccess)
            return noalloc_fail(WB_ERR_CUDA, "wb_vv10_kernel_sum_noalloc: counter", e);
        *pairs_kept = (int64_t)kept;
    }
    return WB_OK;
}
