// Batched fused COSX G kernels of the classes with an f shell (la = 3).
#include "cosx_batch.cuh"

namespace wb {

cudaError_t launch_cosx_f_class_batch(int cls, const CosxArgs* args, const int* off,
                                      int nmol, int* work, int rmax, const int* order,
                                    int grid,
                                      cudaStream_t s, bool far, size_t smem,
                                      bool dual) {
    switch (cls) {
    case 6: return batch_run<3, 0>(args, off, nmol, work, rmax, order, grid, s, far, smem, dual);
    case 7: return batch_run<3, 1>(args, off, nmol, work, rmax, order, grid, s, far, smem, dual);
    case 8: return batch_run<3, 2>(args, off, nmol, work, rmax, order, grid, s, far, smem, dual);
    case 9: return batch_run<3, 3>(args, off, nmol, work, rmax, order, grid, s, far, smem, dual);
    default: return cudaErrorInvalidValue;
    }
}

}  // namespace wb
