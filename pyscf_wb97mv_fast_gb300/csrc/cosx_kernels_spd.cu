// Fused COSX G kernels of the s/p/d classes (la, lb <= 2) and the class
// dispatcher.
#include "cosx_kernels.cuh"

namespace wb {

cudaError_t launch_cosx_f_class(int cls, const CosxArgs& a, int pb, int pe,
                                int grid, cudaStream_t s, bool far);
int cosx_f_class_blocks_per_sm(int cls, bool far);

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

cudaError_t launch_cosx_class_range(int cls, const CosxArgs& a, int pb,
                                    int pe, int grid, cudaStream_t s, bool far) {
    switch (cls) {
    case 0: return run<0, 0>(a, pb, pe, grid, s, far);
    case 1: return run<1, 0>(a, pb, pe, grid, s, far);
    case 2: return run<1, 1>(a, pb, pe, grid, s, far);
    case 3: return run<2, 0>(a, pb, pe, grid, s, far);
    case 4: return run<2, 1>(a, pb, pe, grid, s, far);
    case 5: return run<2, 2>(a, pb, pe, grid, s, far);
    default: return launch_cosx_f_class(cls, a, pb, pe, grid, s, far);
    }
}

int cosx_class_blocks_per_sm(int cls, bool far) {
    switch (cls) {
    case 0: return occ<0, 0>(far);
    case 1: return occ<1, 0>(far);
    case 2: return occ<1, 1>(far);
    case 3: return occ<2, 0>(far);
    case 4: return occ<2, 1>(far);
    case 5: return occ<2, 2>(far);
    default: return cosx_f_class_blocks_per_sm(cls, far);
    }
}

int cosx_class_pts(int cls) {
    switch (cls) {
    case 0: return ClassPts<0, 0>::value;
    case 1: return ClassPts<1, 0>::value;
    case 2: return ClassPts<1, 1>::value;
    case 3: return ClassPts<2, 0>::value;
    case 4: return ClassPts<2, 1>::value;
    case 5: return ClassPts<2, 2>::value;
    case 6: return ClassPts<3, 0>::value;
    case 7: return ClassPts<3, 1>::value;
    case 8: return ClassPts<3, 2>::value;
    default: return ClassPts<3, 3>::value;
    }
}

}  // namespace wb
