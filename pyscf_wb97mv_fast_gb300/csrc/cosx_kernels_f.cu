// Fused COSX G kernels of the classes with an f shell (la = 3).
#include "cosx_kernels.cuh"

namespace wb {

template<int LA, int LB>
static cudaError_t run(const CosxArgs& a, int pb, int pe, int grid,
                       cudaStream_t s) {
    cosx_class_kernel<LA, LB><<<grid, kCtaThreads, 0, s>>>(a, pb, pe);
    return cudaGetLastError();
}

template<int LA, int LB>
static int occ() {
    int n = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(
            &n, cosx_class_kernel<LA, LB>, kCtaThreads, 0) != cudaSuccess)
        return 1;
    return n > 0 ? n : 1;
}

cudaError_t launch_cosx_f_class(int cls, const CosxArgs& a, int pb, int pe,
                                int grid, cudaStream_t s) {
    switch (cls) {
    case 6: return run<3, 0>(a, pb, pe, grid, s);
    case 7: return run<3, 1>(a, pb, pe, grid, s);
    case 8: return run<3, 2>(a, pb, pe, grid, s);
    case 9: return run<3, 3>(a, pb, pe, grid, s);
    default: return cudaErrorInvalidValue;
    }
}

int cosx_f_class_blocks_per_sm(int cls) {
    switch (cls) {
    case 6: return occ<3, 0>();
    case 7: return occ<3, 1>();
    case 8: return occ<3, 2>();
    case 9: return occ<3, 3>();
    default: return 1;
    }
}

}  // namespace wb
