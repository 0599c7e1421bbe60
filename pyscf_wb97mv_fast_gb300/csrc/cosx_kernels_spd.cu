// Fused COSX G kernels of the s/p/d classes (la, lb <= 2) and the class
// dispatcher.
#include "cosx_kernels.cuh"

namespace wb {

cudaError_t launch_cosx_f_class(int cls, const CosxArgs& a, int pb, int pe,
                                int grid, cudaStream_t s, bool far, size_t smem,
                                bool dual);
int cosx_f_class_blocks_per_sm(int cls, bool far, size_t smem, bool dual);

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

cudaError_t launch_cosx_class_range(int cls, const CosxArgs& a, int pb,
                                    int pe, int grid, cudaStream_t s, bool far,
                                    size_t smem, bool dual) {
    switch (cls) {
    case 0: return run<0, 0>(a, pb, pe, grid, s, far, smem, dual);
    case 1: return run<1, 0>(a, pb, pe, grid, s, far, smem, dual);
    case 2: return run<1, 1>(a, pb, pe, grid, s, far, smem, dual);
    case 3: return run<2, 0>(a, pb, pe, grid, s, far, smem, dual);
    case 4: return run<2, 1>(a, pb, pe, grid, s, far, smem, dual);
    case 5: return run<2, 2>(a, pb, pe, grid, s, far, smem, dual);
    default: return launch_cosx_f_class(cls, a, pb, pe, grid, s, far, smem, dual);
    }
}

int cosx_class_blocks_per_sm(int cls, bool far, size_t smem, bool dual) {
    switch (cls) {
    case 0: return occ<0, 0>(far, smem, dual);
    case 1: return occ<1, 0>(far, smem, dual);
    case 2: return occ<1, 1>(far, smem, dual);
    case 3: return occ<2, 0>(far, smem, dual);
    case 4: return occ<2, 1>(far, smem, dual);
    case 5: return occ<2, 2>(far, smem, dual);
    default: return cosx_f_class_blocks_per_sm(cls, far, smem, dual);
    }
}

int cosx_class_pts(int cls, bool dual) {
    switch (cls) {
    case 0: return dual ? ClassPts<0, 0, 2>::value : ClassPts<0, 0>::value;
    case 1: return dual ? ClassPts<1, 0, 2>::value : ClassPts<1, 0>::value;
    case 2: return dual ? ClassPts<1, 1, 2>::value : ClassPts<1, 1>::value;
    case 3: return dual ? ClassPts<2, 0, 2>::value : ClassPts<2, 0>::value;
    case 4: return dual ? ClassPts<2, 1, 2>::value : ClassPts<2, 1>::value;
    case 5: return dual ? ClassPts<2, 2, 2>::value : ClassPts<2, 2>::value;
    case 6: return dual ? ClassPts<3, 0, 2>::value : ClassPts<3, 0>::value;
    case 7: return dual ? ClassPts<3, 1, 2>::value : ClassPts<3, 1>::value;
    case 8: return dual ? ClassPts<3, 2, 2>::value : ClassPts<3, 2>::value;
    default: return dual ? ClassPts<3, 3, 2>::value : ClassPts<3, 3>::value;
    }
}

}  // namespace wb
