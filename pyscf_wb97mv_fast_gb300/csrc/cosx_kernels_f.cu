// Fused COSX G kernels of the classes with an f shell (la = 3).
#include "cosx_kernels.cuh"

namespace wb {

template<int LA, int LB, bool FAR, bool STAGE, int NW = 1>
static cudaError_t run1(const CosxArgs& a, int pb, int pe, int grid,
                        size_t smem, cudaStream_t s) {
    auto k = cosx_class_kernel<LA, LB, FAR, STAGE, NW>;
    if (smem > 48 * 1024) {
        const cudaError_t e = cudaFuncSetAttribute(
            k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
    }
    k<<<grid, kCtaThreads, smem, s>>>(a, pb, pe);
    return cudaGetLastError();
}

template<int LA, int LB>
static cudaError_t run(const CosxArgs& a, int pb, int pe, int grid,
                       cudaStream_t s, bool far, size_t smem, bool dual) {
    if (dual) return run1<LA, LB, false, true, 2>(a, pb, pe, grid, smem, s);
    if (smem)
        return far ? run1<LA, LB, true, true>(a, pb, pe, grid, smem, s)
                   : run1<LA, LB, false, true>(a, pb, pe, grid, smem, s);
    return far ? run1<LA, LB, true, false>(a, pb, pe, grid, 0, s)
               : run1<LA, LB, false, false>(a, pb, pe, grid, 0, s);
}

template<int LA, int LB, bool FAR, bool STAGE, int NW = 1>
static int occ1(size_t smem) {
    auto k = cosx_class_kernel<LA, LB, FAR, STAGE, NW>;
    if (smem > 48 * 1024 &&
        cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)smem) != cudaSuccess)
        return 0;
    int n = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k, kCtaThreads, smem) !=
        cudaSuccess)
        return 0;
    return n;
}

template<int LA, int LB>
static int occ(bool far, size_t smem, bool dual) {
    if (dual) return occ1<LA, LB, false, true, 2>(smem);
    if (smem)
        return far ? occ1<LA, LB, true, true>(smem) : occ1<LA, LB, false, true>(smem);
    return far ? occ1<LA, LB, true, false>(0) : occ1<LA, LB, false, false>(0);
}

cudaError_t launch_cosx_f_class(int cls, const CosxArgs& a, int pb, int pe,
                                int grid, cudaStream_t s, bool far, size_t smem,
                                bool dual) {
    switch (cls) {
    case 6: return run<3, 0>(a, pb, pe, grid, s, far, smem, dual);
    case 7: return run<3, 1>(a, pb, pe, grid, s, far, smem, dual);
    case 8: return run<3, 2>(a, pb, pe, grid, s, far, smem, dual);
    case 9: return run<3, 3>(a, pb, pe, grid, s, far, smem, dual);
    default: return cudaErrorInvalidValue;
    }
}

int cosx_f_class_blocks_per_sm(int cls, bool far, size_t smem, bool dual) {
    switch (cls) {
    case 6: return occ<3, 0>(far, smem, dual);
    case 7: return occ<3, 1>(far, smem, dual);
    case 8: return occ<3, 2>(far, smem, dual);
    case 9: return occ<3, 3>(far, smem, dual);
    default: return 0;
    }
}

}  // namespace wb
