// FP64-accurate GEMMs on bf16 tensor cores (Ozaki split), see ozaki.cu.
#pragma once
#include <cublas_v2.h>
#include <cuda_runtime.h>

#include <cstddef>
#include <cstdint>

namespace wb {

constexpr int kOzSlices = 5;   // 7-bit slices per operand (~35 bits)
constexpr int kOzKc = 768;     // K-GEMM chunk: (l + 1) * Kc < 4096 for l < 5

// the F GEMM needs kOzSlices * nao < 4096 (exact FP32 level sums)
inline bool ozaki_f_supported(int nao) { return kOzSlices * nao < 4096; }

size_t ozaki_f_bytes(int nao, int64_t ld);
size_t ozaki_k_bytes(int nao, int64_t ld);

// F (nao, ld) FP32 AO-major = fl32(X QD); X (nao, ld) FP64 AO-major, QD
// (nao, nao) row-major FP64.  Returns 0, a cudaError_t, or 1000 + cuBLAS
// status.
int ozaki_f_gemm(cublasHandle_t hb, const double* X, const double* QD,
                 int nao, int64_t ld, float* F, void* ws, cudaStream_t s);

// K (nao, nao) row-major (+)= X^T (w o G) over the npts valid points.
int ozaki_k_gemm(cublasHandle_t hb, const double* X, const float* G,
                 const double* w, int nao, int64_t ld, int64_t npts,
                 int accumulate, double* K, void* ws, cudaStream_t s);

}  // namespace wb
