// Device-side pieces of the fused COSX exchange kernel family (sm_103a):
// the per-class task bodies (generated/cosx_classes.cuh).
#pragma once
#include "cosx_args.hpp"
#include "boys.cuh"

namespace wb {

template<int LA, int LB, bool DIAG>
__device__ __forceinline__ void cosx_task(
    const CosxArgs& A, const int4 hdr, const long long g,
    const float gxh, const float gyh, const float gzh,
    const float gxl, const float gyl, const float gzl,
    const float4* __restrict__ stab);

}  // namespace wb

namespace wb {
#include "generated/cosx_classes.cuh"
}
