// The per-(point block, shell pair) screen of the fused G kernels, shared
// with the screen-mask export (aux_kernels.cu) that the superset test reads.
//
// The reference's locked bound (gpu/sgx_k.py:417-456, gpu/shellpairs.py:
// 545-555): tau * sum_prim pref * F0(p' d_min^2) * max(msh_A, msh_B), with
// d_min shrunk by more than its FP32 error and the tolerance divided by
// 1.001 on the host, so the FP32 estimate bounds the FP64 one from above.
#pragma once
#include <cuda_runtime.h>

namespace wb {

// tp = (tau, tau * sum pref), f = max(msh_A, msh_B) of the block; bnd and
// bpref start at the class's first primitive pair (hdr.z is class-local)
__device__ __forceinline__ bool screen_pair(const float tol,
                                            const float4* __restrict__ bnd,
                                            const float* __restrict__ bpref,
                                            const float4 cr, const int4 hdr,
                                            const float2 tp, const float f) {
    // F_0 <= 1: tau * sum(pref) * f bounds the full estimate from above
    if (tp.y * f * 1.0001f < tol) return false;
    const int pp0 = hdr.z, npp = hdr.w & 0xffff;
    float b = 0.0f;
    for (int m = pp0; m < pp0 + npp; ++m) {
        const float4 bp = bnd[m];
        const float dx = bp.x - cr.x, dy = bp.y - cr.y, dz = bp.z - cr.z;
        const float dist = sqrtf(dx * dx + dy * dy + dz * dz);
        float d = dist - cr.w - 1e-5f * (dist + cr.w) - 1e-6f;
        d = fmaxf(d, 0.0f);
        const float T = bp.w * d * d;
        const float f0 = (T > 1e-12f)
            ? 0.88622692545f * erff(sqrtf(T)) * rsqrtf(T) : 1.0f;
        b += bpref[m] * f0;
    }
    return tp.x * b * f >= tol;
}

}  // namespace wb
