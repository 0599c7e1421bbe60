// Batched fused COSX G kernels (several molecules per launch) of the
// s/p/d classes and the batched class dispatcher.
#include "cosx_batch.cuh"

namespace wb {

cudaError_t launch_cosx_class_batch(int cls, const CosxArgs* args, const int* off,
                                    int nmol, int* work, int rmax, const int* order,
                                    int grid,
                                    cudaStream_t s, bool far, size_t smem,
                                    bool dual) {
    switch (cls) {
    case 0: return batch_run<0, 0>(args, off, nmol, work, rmax, order, grid, s, far, smem, dual);
    case 1: return batch_run<1, 0>(args, off, nmol, work, rmax, order, grid, s, far, smem, dual);
    case 2: return batch_run<1, 1>(args, off, nmol, work, rmax, order, grid, s, far, smem, dual);
    case 3: return batch_run<2, 0>(args, off, nmol, work, rmax, order, grid, s, far, smem, dual);
    case 4: return batch_run<2, 1>(args, off, nmol, work, rmax, order, grid, s, far, smem, dual);
    case 5: return batch_run<2, 2>(args, off, nmol, work, rmax, order, grid, s, far, smem, dual);
    default:
        return launch_cosx_f_class_batch(cls, args, off, nmol, work, rmax, order, grid,
                                         s, far, smem, dual);
    }
}

}  // namespace wb
