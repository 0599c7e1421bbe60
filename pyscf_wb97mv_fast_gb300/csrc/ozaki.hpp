// FP64-accurate GEMMs on bf16 tensor cores (Ozaki split), see ozaki.cu.
#pragma once
#include <cublas_v2.h>
#include <cuda_runtime.h>

#include <cstddef>
#include <cstdint>

namespace wb {

constexpr int kOzBits = 6;     // balanced digits, |d| <= 32
constexpr int kOzSlices = 7;   // 42 bits per operand
constexpr int kOzKc = 2048;    // K-GEMM chunk: (l + 1) * Kc < 2^14 for l < 7

// exact FP32 level sums need kOzSlices * K < 2^14 along the inner dimension
inline bool ozaki_f_supported(int nao) { return kOzSlices * nao < (1 << 14); }

size_t ozaki_f_bytes(int nao, int64_t ld);
// workspace of the K split for nrhs right-hand sides (w o G of several
// omegas against the same X)
size_t ozaki_k_bytes(int nao, int64_t ld, int nrhs = 1);

// F (nao, ld) FP32 AO-major = fl32(X QD); X (nao, ld) FP64 AO-major, QD
// (nao, nao) row-major FP64.  Returns 0, a cudaError_t, or 1000 + cuBLAS
// status.  status (optional, device): bit 0 is set when a wait of the
// tensor-core kernel gave up (the affected F entries are NaN).
int ozaki_f_gemm(cublasHandle_t hb, const double* X, const double* QD,
                 int nao, int64_t ld, float* F, void* ws, cudaStream_t s,
                 unsigned long long* status = nullptr);

// the same product with FP64 output: the combined level sums (42 bits
// relative to the per-point / per-column maxima) rounded once to FP64
int ozaki_f_gemm64(cublasHandle_t hb, const double* X, const double* QD,
                   int nao, int64_t ld, double* F, void* ws, cudaStream_t s,
                   unsigned long long* status = nullptr);

// K (+)= X^T (w o G) with G FP64 (w o G formed in FP64 before the split)
int ozaki_k_gemm64(cublasHandle_t hb, const double* X, const double* G,
                   const double* w, int nao, int64_t ld, int64_t npts,
                   int accumulate, double* K, void* ws, cudaStream_t s);

// the two engines of the F product (bitwise the same F): cuBLAS level
// GEMMs (the default) and this library's tcgen05 kernel
constexpr int kOzEngineLibrary = 0;
constexpr int kOzEngineTc = 1;
void ozaki_set_f_engine(int engine);
int ozaki_get_f_engine();
// this library's kernel launches of one F product under the current engine
inline int ozaki_f_launches() { return ozaki_get_f_engine() == kOzEngineTc ? 4 : 4 + kOzSlices; }
int ozaki_f_gemm_cublas(cublasHandle_t hb, const double* X, const double* QD,
                        int nao, int64_t ld, float* F, void* ws, cudaStream_t s);
int ozaki_f_gemm_tc(const double* X, const double* QD, int nao, int64_t ld, float* F,
                    void* ws, cudaStream_t s, unsigned long long* status);
int ozaki_f_gemm_cublas64(cublasHandle_t hb, const double* X, const double* QD,
                          int nao, int64_t ld, double* F, void* ws, cudaStream_t s);
int ozaki_f_gemm_tc64(const double* X, const double* QD, int nao, int64_t ld, double* F,
                      void* ws, cudaStream_t s, unsigned long long* status);
size_t ozaki_f_tc_bytes(int nao, int64_t ld);
// exponent of max_l |X(l, g)| per point g (shared by both engines)
void f_rowmax(const double* X, int nao, int64_t ld, int* erow, cudaStream_t s);

// K (nao, nao) row-major (+)= X^T (w o G) over the npts valid points.
// x_sliced: ws already holds the slices of this X (an earlier call on the
// same X and workspace, e.g. another omega of the same tile), which are
// reused.
int ozaki_k_gemm(cublasHandle_t hb, const double* X, const float* G,
                 const double* w, int nao, int64_t ld, int64_t npts,
                 int accumulate, double* K, void* ws, cudaStream_t s,
                 bool x_sliced = false);

// K_r (+)= X^T (w o G_r) for r < nrhs (<= 8) in one split: X sliced once,
// the w o G_r side by side (N = nrhs nao per level GEMM), one combine.
int ozaki_k_gemm_multi(cublasHandle_t hb, const double* X, const float* const* G,
                       int nrhs, const double* w, int nao, int64_t ld,
                       int64_t npts, int accumulate, double* const* K, void* ws,
                       cudaStream_t s, bool x_sliced = false);

}  // namespace wb
