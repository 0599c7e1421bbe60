// Fused screen + G kernel of one shell-pair class (included by the
// cosx_kernels_*.cu translation units, which pick the classes).
//
// One warp owns one 32-point sub-block at a time (one grid point per lane)
// and walks the class's shell pairs in ascending (A, B) order: 32 pairs at
// a time every lane loads one pair header and evaluates its screening
// bound, a ballot compacts the kept ones, and the warp then runs each kept
// task with all lanes (headers by shuffle, the next task's F_B prefetched
// while the current one computes).  Tasks with the same bra shell A form a
// run: F_A is read and G_A written once per run.  A warp takes the next
// sub-block from a per-class counter (dynamic load balance); every G
// element is written by exactly one lane in a fixed order, so results do
// not depend on the launch shape or scheduling.
//
// The bound is the reference's locked estimate (gpu/sgx_k.py:35-46,
// :417-456): tau * sum_prim pref F_0(p' d_min^2) * max(msh_A, msh_B) with
// d_min shrunk by 1e-5 (d + r) + 1e-6 and tol already divided by 1.001.
#pragma once
#include "launch.hpp"
#include "cosx_device.cuh"

namespace wb {

constexpr int kCtaThreads = 128;
constexpr int kBoysFloat4 = 145 * 5;

__device__ __forceinline__ bool screen_pair(const CosxArgs& A, int sub, int k,
                                            const float4 cr, const int4 hdr) {
    const int2 sh = A.pshell[k];
    const float* ms = A.msh + (long long)sub * A.nvshell;
    const float f = fmaxf(ms[sh.x], ms[sh.y]);
    const float2 tp = A.ptau[k];
    // F_0 <= 1: tau * sum(pref) * f bounds the full estimate from above
    if (tp.y * f * 1.0001f < A.tol) return false;
    const int pp0 = hdr.z, npp = hdr.w & 0xffff;
    float b = 0.0f;
    for (int m = pp0; m < pp0 + npp; ++m) {
        const float4 bp = A.bnd[m];
        const float dx = bp.x - cr.x, dy = bp.y - cr.y, dz = bp.z - cr.z;
        const float dist = sqrtf(dx * dx + dy * dy + dz * dz);
        float d = dist - cr.w - 1e-5f * (dist + cr.w) - 1e-6f;
        d = fmaxf(d, 0.0f);
        const float T = bp.w * d * d;
        const float f0 = (T > 1e-12f)
            ? 0.88622692545f * erff(sqrtf(T)) * rsqrtf(T) : 1.0f;
        b += A.bpref[m] * f0;
    }
    return tp.x * b * f >= A.tol;
}

__device__ __forceinline__ int4 shfl_int4(const int4 v, int src) {
    return make_int4(__shfl_sync(0xffffffffu, v.x, src),
                     __shfl_sync(0xffffffffu, v.y, src),
                     __shfl_sync(0xffffffffu, v.z, src),
                     __shfl_sync(0xffffffffu, v.w, src));
}

template<int LB>
__device__ __forceinline__ void load_fb(const CosxArgs& A, const int ib0,
                                        const long long g, float* fb) {
#pragma unroll
    for (int nu = 0; nu < 2 * LB + 1; ++nu)
        fb[nu] = A.F[(long long)(ib0 + nu) * A.ld + g];
}

template<int LA, int LB>
__global__ void __launch_bounds__(kCtaThreads)
cosx_class_kernel(const CosxArgs A, const int pair_begin, const int pair_end) {
    constexpr int CLS = LA * (LA + 1) / 2 + LB;
    constexpr int NCA = (LA + 1) * (LA + 2) / 2;
    constexpr int NB = 2 * LB + 1;
    __shared__ float4 stab[kBoysFloat4];
    for (int i = threadIdx.x; i < kBoysFloat4; i += blockDim.x)
        stab[i] = A.boys[i];
    __syncthreads();
    const int lane = threadIdx.x & 31;
    unsigned long long kept = 0, flops = 0, ints = 0;
    for (;;) {
        int sub = 0;
        if (lane == 0) sub = atomicAdd(A.work + CLS, 1);
        sub = __shfl_sync(0xffffffffu, sub, 0);
        if (sub >= A.nsub) break;
        const long long g = (long long)sub * 32 + lane;
        const float gxh = A.gxyz_hi[g], gyh = A.gxyz_hi[A.ld + g],
                    gzh = A.gxyz_hi[2 * A.ld + g];
        const float gxl = A.gxyz_lo[g], gyl = A.gxyz_lo[A.ld + g],
                    gzl = A.gxyz_lo[2 * A.ld + g];
        const float4 cr = A.sub_cr[sub];
        const int nvalid = min(32, A.npts - sub * 32);
        // run state: the current bra shell (its first AO), f0 and Xa
        int curA = -1;
        float f0[NCA], Xa[NCA];
#pragma unroll
        for (int c = 0; c < NCA; ++c) { f0[c] = 0.0f; Xa[c] = 0.0f; }
        for (int c0 = pair_begin; c0 < pair_end; c0 += 32) {
            // every lane fetches one pair header: the screen uses it, and
            // the kept tasks get theirs by shuffle (no dependent load)
            const int k = c0 + lane;
            bool keep = k < pair_end;
            int4 hl = make_int4(0, 0, 0, 0);
            if (keep) hl = A.hdr[k];
            if (keep && A.tol > 0.0f) keep = screen_pair(A, sub, k, cr, hl);
            unsigned mask = __ballot_sync(0xffffffffu, keep);
            if (!mask) continue;
            int j = __ffs(mask) - 1;
            int4 hdr = shfl_int4(hl, j);
            float fb[NB];
            load_fb<LB>(A, hdr.y, g, fb);
            while (true) {
                mask &= mask - 1;
                // prefetch the next kept task of this chunk
                const bool more = mask != 0u;
                int4 hn = hdr;
                float fbn[NB];
                if (more) {
                    hn = shfl_int4(hl, __ffs(mask) - 1);
                    load_fb<LB>(A, hn.y, g, fbn);
                }
                if (hdr.x != curA) {
                    if (curA >= 0) cosx_end<LA>(A, curA, g, Xa);
                    curA = hdr.x;
                    cosx_begin<LA>(A, curA, g, f0);
#pragma unroll
                    for (int c = 0; c < NCA; ++c) Xa[c] = 0.0f;
                }
                if constexpr (LA == LB) {
                    if (hdr.w >> 16)
                        cosx_task<LA, LB, true>(A, hdr, g, gxh, gyh, gzh, gxl,
                                                gyl, gzl, stab, f0, fb, Xa);
                    else
                        cosx_task<LA, LB, false>(A, hdr, g, gxh, gyh, gzh, gxl,
                                                 gyl, gzl, stab, f0, fb, Xa);
                } else {
                    cosx_task<LA, LB, false>(A, hdr, g, gxh, gyh, gzh, gxl,
                                             gyl, gzl, stab, f0, fb, Xa);
                }
                if (lane == 0) {
                    // hdr.w holds npp | diag << 16; pair index from lane j
                    kept += 1;
                }
                if (!more) break;
                hdr = hn;
#pragma unroll
                for (int nu = 0; nu < NB; ++nu) fb[nu] = fbn[nu];
            }
            // model flops / integrals of the kept tasks of this chunk
            const unsigned km = __ballot_sync(0xffffffffu, keep);
            if (keep) {
                const unsigned long long fl = (unsigned long long)A.pflops[k] * nvalid;
                const unsigned long long it = (unsigned long long)A.pnint[k] * nvalid;
                flops += fl;
                ints += it;
            }
            (void)km;
        }
        if (curA >= 0) cosx_end<LA>(A, curA, g, Xa);
    }
    // lane 0 counted the tasks, every lane its own pairs' flops / integrals
    for (int o = 16; o > 0; o >>= 1) {
        flops += __shfl_xor_sync(0xffffffffu, flops, o);
        ints += __shfl_xor_sync(0xffffffffu, ints, o);
    }
    if (lane == 0 && kept) {
        atomicAdd(A.counters + 3 * CLS + 0, kept);
        atomicAdd(A.counters + 3 * CLS + 1, flops);
        atomicAdd(A.counters + 3 * CLS + 2, ints);
    }
}

}  // namespace wb
