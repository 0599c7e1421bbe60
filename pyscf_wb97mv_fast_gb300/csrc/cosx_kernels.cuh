// Fused screen + G kernel of one shell-pair class (included by the
// cosx_kernels_*.cu translation units, which pick the classes).
//
// One warp owns one 32-point sub-block at a time (one grid point per lane)
// and walks the class's shell pairs in ascending order: 32 pairs at a time
// every lane evaluates the screening bound of one pair, a ballot compacts
// the kept ones, and the warp then runs each kept task with all lanes.  A
// warp takes the next sub-block from a per-class counter (dynamic load
// balance); every G element is written by exactly one lane in a fixed
// order, so results do not depend on the launch shape or scheduling.
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
                                            const float4 cr) {
    const int2 sh = A.pshell[k];
    const float* ms = A.msh + (long long)sub * A.nvshell;
    const float f = fmaxf(ms[sh.x], ms[sh.y]);
    const float2 tp = A.ptau[k];
    // F_0 <= 1: tau * sum(pref) * f bounds the full estimate from above
    if (tp.y * f * 1.0001f < A.tol) return false;
    const int4 hdr = A.hdr[k];
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

template<int LA, int LB>
__global__ void __launch_bounds__(kCtaThreads)
cosx_class_kernel(const CosxArgs A, const int pair_begin, const int pair_end) {
    constexpr int CLS = LA * (LA + 1) / 2 + LB;
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
        for (int c0 = pair_begin; c0 < pair_end; c0 += 32) {
            const int k = c0 + lane;
            bool keep = k < pair_end;
            if (keep && A.tol > 0.0f) keep = screen_pair(A, sub, k, cr);
            unsigned mask = __ballot_sync(0xffffffffu, keep);
            while (mask) {
                const int j = __ffs(mask) - 1;
                mask &= mask - 1;
                const int kk = c0 + j;
                const int4 hdr = A.hdr[kk];
                if constexpr (LA == LB) {
                    if (hdr.w >> 16)
                        cosx_task<LA, LB, true>(A, hdr, g, gxh, gyh, gzh,
                                                gxl, gyl, gzl, stab);
                    else
                        cosx_task<LA, LB, false>(A, hdr, g, gxh, gyh, gzh,
                                                 gxl, gyl, gzl, stab);
                } else {
                    cosx_task<LA, LB, false>(A, hdr, g, gxh, gyh, gzh,
                                             gxl, gyl, gzl, stab);
                }
                if (lane == 0) {
                    kept += 1;
                    flops += (unsigned long long)A.pflops[kk] * nvalid;
                    ints += (unsigned long long)A.pnint[kk] * nvalid;
                }
            }
        }
    }
    if (lane == 0 && kept) {
        atomicAdd(A.counters + 3 * CLS + 0, kept);
        atomicAdd(A.counters + 3 * CLS + 1, flops);
        atomicAdd(A.counters + 3 * CLS + 2, ints);
    }
}

}  // namespace wb
