// Fused COSX G kernels of the classes with an f shell (la = 3).
#include "cosx_kernels.cuh"

namespace wb {

template<int LA, int LB>
static cudaError_t run(const CosxArgs& a, int pb, int pe, int grid,
                       cudaStream_t s, bool far) {
    if (far)
        cosx_class_kernel<LA, LB, true><<<grid, kCtaThreads, 0, s>>>(a, pb, pe);
    else
        cosx_class_kernel<LA, LB, false><<<grid, kCtaThreads, 0, s>>>(a, pb, pe);
    return cudaGetLastError();
}

template<int LA, int LB>
static int occ(bool far) {
    int n = 0;
    const cudaError_t e = far
        ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(
              &n, cosx_class_kernel<LA, LB, true>, kCtaThreads, 0)
        : cudaOccupancyMaxActiveBlocksPerMultiprocessor(
              &n, cosx_class_kernel<LA, LB, false>, kCtaThreads, 0);
    if (e != cudaSuccess) return 1;
    return n > 0 ? n : 1;
}

cudaError_t launch_cosx_f_class(int cls, const CosxArgs& a, int pb, int pe,
                                int grid, cudaStream_t s, bool far) {
    switch (cls) {
    case 6: return run<3, 0>(a, pb, pe, grid, s, far);
    case 7: return run<3, 1>(a, pb, pe, grid, s, far);
    case 8: return run<3, 2>(a, pb, pe, grid, s, far);
    case 9: return run<3, 3>(a, pb, pe, grid, s, far);
    default: return cudaErrorInvalidValue;
    }
}

int cosx_f_class_blocks_per_sm(int cls, bool far) {
    switch (cls) {
    case 6: return occ<3, 0>(far);
    case 7: return occ<3, 1>(far);
    case 8: return occ<3, 2>(far);
    case 9: return occ<3, 3>(far);
    default: return 1;
    }
}

}  // namespace wb
