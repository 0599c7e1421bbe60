// Plain FP64 form of the fused screen + G kernels: the f classes (their
// own translation unit, compiled in parallel with the others).
#include "cosx_fp64.cuh"

namespace wb {

cudaError_t launch_cosx_fp64_f(int cls, const CosxF64Args& a, int pb, int pe, int nsm,
                               cudaStream_t s) {
    switch (cls) {
    case 6: return f64::run64<3, 0>(a, cls, pb, pe, nsm, s);
    case 7: return f64::run64<3, 1>(a, cls, pb, pe, nsm, s);
    case 8: return f64::run64<3, 2>(a, cls, pb, pe, nsm, s);
    case 9: return f64::run64<3, 3>(a, cls, pb, pe, nsm, s);
    default: return cudaErrorInvalidValue;
    }
}

}  // namespace wb
