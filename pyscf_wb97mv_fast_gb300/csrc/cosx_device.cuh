// Device-side pieces of the fused COSX exchange kernel family (sm_103a):
// the per-class task bodies (generated/cosx_classes.cuh).
#pragma once
#include "cosx_args.hpp"
#include "boys.cuh"

namespace wb {

// One task of class (LA, LB): primitive-pair loop, G_B update, bra-side
// Cartesian accumulators Xa carried across the run of tasks with the same A.
template<int LA, int LB, bool DIAG>
__device__ __forceinline__ void cosx_task(
    const CosxArgs& A, const int4 hdr, const long long g,
    const float gxh, const float gyh, const float gzh,
    const float gxl, const float gyl, const float gzl,
    const float4* __restrict__ stab, const float* f0, const float* fb,
    float* Xa);

// Start of a run: f0 = c2s^T F_A (Cartesian components of F on shell A).
template<int LA>
__device__ __forceinline__ void cosx_begin(const CosxArgs& A, const int ia0,
                                           const long long g, float* f0);

// End of a run: G_A += c2s^T Xa.
template<int LA>
__device__ __forceinline__ void cosx_end(const CosxArgs& A, const int ia0,
                                         const long long g, const float* Xa);

}  // namespace wb

namespace wb {
#include "generated/cosx_classes.cuh"
}
