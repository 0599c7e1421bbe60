// Plain FP64 form of the fused screen + G kernels: the s/p/d classes, the
// class dispatcher and the FP64 weight pass (the kernel itself is in
// cosx_fp64.cuh).
#include "cosx_fp64.cuh"

namespace wb {

cudaError_t launch_cosx_fp64_class(int cls, const CosxF64Args& a, int pb, int pe,
                                   int nsm, cudaStream_t s) {
    switch (cls) {
    case 0: return f64::run64<0, 0>(a, cls, pb, pe, nsm, s);
    case 1: return f64::run64<1, 0>(a, cls, pb, pe, nsm, s);
    case 2: return f64::run64<1, 1>(a, cls, pb, pe, nsm, s);
    case 3: return f64::run64<2, 0>(a, cls, pb, pe, nsm, s);
    case 4: return f64::run64<2, 1>(a, cls, pb, pe, nsm, s);
    case 5: return f64::run64<2, 2>(a, cls, pb, pe, nsm, s);
    default: return launch_cosx_fp64_f(cls, a, pb, pe, nsm, s);
    }
}

namespace {
__global__ void weight_g64_kernel(const double* __restrict__ G,
                                  const double* __restrict__ w, int64_t npts,
                                  int64_t ld, int nao, double* __restrict__ out) {
    const int64_t n = (int64_t)nao * ld;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x) {
        const int64_t g = i % ld;
        out[i] = g < npts ? w[g] * G[i] : 0.0;
    }
}
}  // namespace

cudaError_t launch_weight_g64(const double* G, const double* w, int64_t npts,
                              int64_t ld, int nao, double* out, cudaStream_t s) {
    const int64_t n = (int64_t)nao * ld;
    const int64_t blocks = grid_stride_blocks(n, 256, 32);
    weight_g64_kernel<<<(int)std::max<int64_t>(blocks, 1), 256, 0, s>>>(G, w, npts, ld,
                                                                      nao, out);
    return cudaGetLastError();
}

}  // namespace wb
