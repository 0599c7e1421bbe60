// Launch helper of the batched class kernels (cosx_batch_spd.cu,
// cosx_batch_f.cu): the variant a class runs (two-omega, staged far / near,
// register-prefetch far / near), as in the single-molecule dispatch.
#pragma once
#include "cosx_kernels.cuh"

namespace wb {

cudaError_t launch_cosx_f_class_batch(int cls, const CosxArgs* args, const int* off,
                                      int nmol, int* work, int rmax, const int* order,
                                      int grid, cudaStream_t s, bool far, size_t smem,
                                      bool dual);

template<int LA, int LB, bool FAR, bool STAGE, int NW = 1>
static cudaError_t batch_run1(const CosxArgs* args, const int* off, int nmol,
                              int* work, int rmax, const int* order, int grid,
                              size_t smem, cudaStream_t s) {
    auto k = cosx_class_kernel_batch<LA, LB, FAR, STAGE, NW>;
    if (smem > 48 * 1024) {
        const cudaError_t e = cudaFuncSetAttribute(
            k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
    }
    k<<<grid, kCtaThreads, smem, s>>>(args, off, nmol, work, rmax, order);
    return cudaGetLastError();
}

template<int LA, int LB>
static cudaError_t batch_run(const CosxArgs* args, const int* off, int nmol,
                             int* work, int rmax, const int* order, int grid,
                             cudaStream_t s, bool far, size_t smem, bool dual) {
    if (dual)
        return batch_run1<LA, LB, false, true, 2>(args, off, nmol, work, rmax, order,
                                                  grid, smem, s);
    if (smem)
        return far ? batch_run1<LA, LB, true, true>(args, off, nmol, work, rmax, order,
                                                    grid, smem, s)
                   : batch_run1<LA, LB, false, true>(args, off, nmol, work, rmax, order,
                                                     grid, smem, s);
    return far ? batch_run1<LA, LB, true, false>(args, off, nmol, work, rmax, order,
                                                 grid, 0, s)
               : batch_run1<LA, LB, false, false>(args, off, nmol, work, rmax, order,
                                                  grid, 0, s);
}

}  // namespace wb
