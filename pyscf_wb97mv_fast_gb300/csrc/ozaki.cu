// FP64-accurate GEMMs of the COSX K build on the bf16 tensor cores.
//
// GB300 runs FP64 at ~1 TFLOP/s, so F = X QD and K = X^T (w o G) -- the
// two dense contractions the reference keeps in FP64 (gpu/sgx_k.py:14-28,
// :722, :734) -- would dominate the build.  They run here as an Ozaki
// split (K. Ozaki et al., Numer. Algorithms 59 (2012) 95-118; on tensor
// cores: H. Ootomo, K. Ozaki, R. Yokota, IJHPCA 2024):
//
//   x = 2^e sum_i d_i 2^(-6-7i),   d_i integer in [-64, 64]   (bf16-exact)
//
// with e per row / column (chunk), digits by round-to-nearest, s slices.
// A product level l = i + j collects sum_{i+j=l} A_i B_j in ONE bf16 GEMM
// with FP32 accumulation: storing the A slices ascending and the B slices
// descending along K makes every level a prefix of A times a suffix of B.
// Every product is an integer of magnitude <= 2^12 and a level sums at most
// (l+1) * Kc of them, so with (l+1) Kc <= 4096 every partial sum is an
// integer below 2^24: the FP32 accumulation is exact, whatever order the
// tensor cores use.  Levels are combined in FP64 (ldexp, exact scaling).
// The result carries ~7s bits relative to the per-row/column maxima; the
// truncated products (i + j >= s) are below 2^(-7s) of them.
//
// The bf16 GEMMs themselves are plain library GEMMs (cuBLAS, bf16 in, FP32
// accumulate); the slicing, the per-chunk scaling and the FP64 level
// combination are this file's kernels.
#include <cublas_v2.h>
#include <cuda_bf16.h>

#include <cmath>
#include <cstdint>

#include "ozaki.hpp"

namespace wb {

__device__ __forceinline__ int exp_of_max(double m) {
    // smallest e with m < 2^e (0 for m == 0)
    if (!(m > 0.0)) return 0;
    int e;
    frexp(m, &e);          // m = f 2^e, f in [0.5, 1)
    return e;
}

// digits of x (|x| < 2^e) -> s values in [-64, 64]
template<int S>
__device__ __forceinline__ void digits(double x, int e, float* d) {
    double r = ldexp(x, 6 - e);                 // |r| < 64
#pragma unroll
    for (int i = 0; i < S; ++i) {
        const double q = rint(r);
        d[i] = (float)q;
        r = (r - q) * 128.0;
    }
}

// ---------------------------------------------------------------------------
// F = X QD.  X (nao, ld) AO-major = column-major A (ld x nao) scaled per row
// g; QD row-major = column-major Q (nao x nao) with Q(mu, l) = QD(l, mu);
// B = Q^T scaled per column mu (= per row mu of Q).
// A_all (ld x S*nao, col-major): column block i = slice i.
// B_all (S*nao x nao, col-major): row block r = slice S-1-r.
// ---------------------------------------------------------------------------
template<int S>
__global__ void f_slice_x_kernel(const double* __restrict__ X, int nao,
                                 int64_t ld, int* __restrict__ erow,
                                 __nv_bfloat16* __restrict__ A) {
    const int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= ld) return;
    double m = 0.0;
    for (int l = 0; l < nao; ++l) m = fmax(m, fabs(X[(int64_t)l * ld + g]));
    const int e = exp_of_max(m);
    erow[g] = e;
    for (int l = 0; l < nao; ++l) {
        float d[S];
        digits<S>(X[(int64_t)l * ld + g], e, d);
#pragma unroll
        for (int i = 0; i < S; ++i)
            A[((int64_t)i * nao + l) * ld + g] = __float2bfloat16_rn(d[i]);
    }
}

template<int S>
__global__ void f_slice_qd_kernel(const double* __restrict__ QD, int nao,
                                  int* __restrict__ ecol,
                                  __nv_bfloat16* __restrict__ B) {
    // one block per column mu of B = Q^T, i.e. QD(:, mu)
    const int mu = blockIdx.x;
    __shared__ double red[256];
    double m = 0.0;
    for (int l = threadIdx.x; l < nao; l += blockDim.x)
        m = fmax(m, fabs(QD[(int64_t)l * nao + mu]));
    red[threadIdx.x] = m;
    __syncthreads();
    for (int s = blockDim.x / 2; s > 0; s >>= 1) {
        if (threadIdx.x < s) red[threadIdx.x] = fmax(red[threadIdx.x], red[threadIdx.x + s]);
        __syncthreads();
    }
    const int e = exp_of_max(red[0]);
    if (threadIdx.x == 0) ecol[mu] = e;
    const int64_t ldb = (int64_t)S * nao;
    for (int l = threadIdx.x; l < nao; l += blockDim.x) {
        float d[S];
        digits<S>(QD[(int64_t)l * nao + mu], e, d);
#pragma unroll
        for (int i = 0; i < S; ++i)
            B[(int64_t)mu * ldb + (int64_t)(S - 1 - i) * nao + l] =
                __float2bfloat16_rn(d[i]);
    }
}

// F32[mu, g] = fl32( sum_l C_l[mu, g] 2^(e_g + f_mu - 12 - 7 l) )
template<int S>
__global__ void f_combine_kernel(const float* __restrict__ C, int nao,
                                 int64_t ld, const int* __restrict__ erow,
                                 const int* __restrict__ ecol,
                                 float* __restrict__ F) {
    const int64_t plane = (int64_t)nao * ld;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < plane;
         i += (int64_t)gridDim.x * blockDim.x) {
        const int64_t mu = i / ld, g = i - mu * ld;
        const int base = erow[g] + ecol[mu] - 12;
        double acc = 0.0;
#pragma unroll
        for (int l = S - 1; l >= 0; --l)
            acc += ldexp((double)C[(int64_t)l * plane + i], base - 7 * l);
        F[i] = __double2float_rn(acc);
    }
}

// ---------------------------------------------------------------------------
// K = X^T (w o G), K dimension = grid points, chunked by KC points with a
// scale per (chunk, column).  Per chunk c, A_c(k, mu) = X[mu, c KC + k] and
// B_c(k, nu) = w_k G[nu, c KC + k]; layouts (col-major, ld = S KC):
//   A: column mu = [slice 0 (KC) | slice 1 | ... ]     (ascending)
//   B: column nu = [slice S-1 | ... | slice 0]          (descending)
// chunk stride S KC nao.  One CTA per (chunk, column), KC threads.
// ---------------------------------------------------------------------------
template<int S, int KC>
__global__ void k_slice_kernel(const double* __restrict__ X,
                               const float* __restrict__ G,
                               const double* __restrict__ w, int nao,
                               int64_t ld, int64_t npts, int nchunk,
                               int* __restrict__ ex, int* __restrict__ ew,
                               __nv_bfloat16* __restrict__ A,
                               __nv_bfloat16* __restrict__ B) {
    const int c = blockIdx.x, col = blockIdx.y;
    const int k = threadIdx.x;
    const int64_t g = (int64_t)c * KC + k;
    __shared__ double rx[KC], rw[KC];
    double xv = 0.0, wv = 0.0;
    if (g < npts) {
        xv = X[(int64_t)col * ld + g];
        wv = w[g] * (double)G[(int64_t)col * ld + g];
    }
    rx[k] = fabs(xv);
    rw[k] = fabs(wv);
    __syncthreads();
    for (int s = KC / 2; s > 0; s >>= 1) {
        if (k < s) {
            rx[k] = fmax(rx[k], rx[k + s]);
            rw[k] = fmax(rw[k], rw[k + s]);
        }
        __syncthreads();
    }
    const int e1 = exp_of_max(rx[0]), e2 = exp_of_max(rw[0]);
    if (k == 0) {
        ex[(int64_t)c * nao + col] = e1;
        ew[(int64_t)c * nao + col] = e2;
    }
    float d1[S], d2[S];
    digits<S>(xv, e1, d1);
    digits<S>(wv, e2, d2);
    const int64_t colbase = (int64_t)c * S * KC * nao + (int64_t)col * S * KC;
#pragma unroll
    for (int i = 0; i < S; ++i) {
        A[colbase + (int64_t)i * KC + k] = __float2bfloat16_rn(d1[i]);
        B[colbase + (int64_t)(S - 1 - i) * KC + k] = __float2bfloat16_rn(d2[i]);
    }
}

// K[mu, nu] (+)= sum_c sum_l C[l][c](mu, nu) 2^(ex[c,mu] + ew[c,nu] - 12 - 7l)
template<int S>
__global__ void k_combine_kernel(const float* __restrict__ C, int nao,
                                 int nchunk, const int* __restrict__ ex,
                                 const int* __restrict__ ew, int accumulate,
                                 double* __restrict__ K) {
    const int64_t n2 = (int64_t)nao * nao;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n2;
         i += (int64_t)gridDim.x * blockDim.x) {
        const int mu = (int)(i % nao), nu = (int)(i / nao);   // C col-major
        double acc = 0.0;
        for (int c = 0; c < nchunk; ++c) {
            const int base = ex[(int64_t)c * nao + mu] + ew[(int64_t)c * nao + nu] - 12;
            double lv = 0.0;
#pragma unroll
            for (int l = S - 1; l >= 0; --l)
                lv += ldexp((double)C[((int64_t)l * nchunk + c) * n2 + i], base - 7 * l);
            acc += lv;
        }
        const int64_t o = (int64_t)mu * nao + nu;              // K row-major
        K[o] = accumulate ? K[o] + acc : acc;
    }
}

// ---------------------------------------------------------------------------
static inline size_t al(size_t x) { return (x + 255) & ~(size_t)255; }

size_t ozaki_f_bytes(int nao, int64_t ld) {
    const size_t S = kOzSlices;
    return al(sizeof(int) * ld) + al(sizeof(int) * nao) +
           al(sizeof(__nv_bfloat16) * S * nao * ld) +
           al(sizeof(__nv_bfloat16) * S * nao * nao) +
           al(sizeof(float) * S * nao * ld);
}

size_t ozaki_k_bytes(int nao, int64_t ld) {
    const size_t S = kOzSlices;
    const int64_t nchunk = (ld + kOzKc - 1) / kOzKc;
    return 2 * al(sizeof(int) * nchunk * nao) +
           2 * al(sizeof(__nv_bfloat16) * S * kOzKc * nchunk * nao) +
           al(sizeof(float) * S * nchunk * (size_t)nao * nao);
}

#define OZ_CUBLAS(call)                                        \
    do {                                                       \
        cublasStatus_t st_ = (call);                           \
        if (st_ != CUBLAS_STATUS_SUCCESS) return (int)st_ + 1000; \
    } while (0)
#define OZ_CUDA(call)                                          \
    do {                                                       \
        cudaError_t e_ = (call);                               \
        if (e_ != cudaSuccess) return (int)e_;                 \
    } while (0)

int ozaki_f_gemm(cublasHandle_t hb, const double* X, const double* QD,
                 int nao, int64_t ld, float* F, void* ws, cudaStream_t s) {
    constexpr int S = kOzSlices;
    char* p = static_cast<char*>(ws);
    int* erow = reinterpret_cast<int*>(p); p += al(sizeof(int) * ld);
    int* ecol = reinterpret_cast<int*>(p); p += al(sizeof(int) * nao);
    __nv_bfloat16* A = reinterpret_cast<__nv_bfloat16*>(p);
    p += al(sizeof(__nv_bfloat16) * (size_t)S * nao * ld);
    __nv_bfloat16* B = reinterpret_cast<__nv_bfloat16*>(p);
    p += al(sizeof(__nv_bfloat16) * (size_t)S * nao * nao);
    float* C = reinterpret_cast<float*>(p);
    f_slice_x_kernel<S><<<(unsigned)((ld + 127) / 128), 128, 0, s>>>(X, nao, ld, erow, A);
    OZ_CUDA(cudaGetLastError());
    f_slice_qd_kernel<S><<<nao, 256, 0, s>>>(QD, nao, ecol, B);
    OZ_CUDA(cudaGetLastError());
    const float one = 1.0f, zero = 0.0f;
    for (int l = 0; l < S; ++l) {
        // C_l (ld x nao) = A[:, 0:(l+1) nao] * B[(S-1-l) nao : S nao, :]
        OZ_CUBLAS(cublasGemmEx(hb, CUBLAS_OP_N, CUBLAS_OP_N, (int)ld, nao,
                               (l + 1) * nao, &one, A, CUDA_R_16BF, (int)ld,
                               B + (size_t)(S - 1 - l) * nao, CUDA_R_16BF,
                               S * nao, &zero, C + (size_t)l * nao * ld,
                               CUDA_R_32F, (int)ld, CUBLAS_COMPUTE_32F,
                               CUBLAS_GEMM_DEFAULT));
    }
    const int64_t plane = (int64_t)nao * ld;
    int64_t blocks = (plane + 255) / 256;
    if (blocks > 152 * 32) blocks = 152 * 32;
    f_combine_kernel<S><<<(unsigned)blocks, 256, 0, s>>>(C, nao, ld, erow, ecol, F);
    OZ_CUDA(cudaGetLastError());
    return 0;
}

int ozaki_k_gemm(cublasHandle_t hb, const double* X, const float* G,
                 const double* w, int nao, int64_t ld, int64_t npts,
                 int accumulate, double* K, void* ws, cudaStream_t s) {
    constexpr int S = kOzSlices, KC = kOzKc;
    const int nchunk = (int)((ld + KC - 1) / KC);
    char* p = static_cast<char*>(ws);
    int* ex = reinterpret_cast<int*>(p); p += al(sizeof(int) * (size_t)nchunk * nao);
    int* ew = reinterpret_cast<int*>(p); p += al(sizeof(int) * (size_t)nchunk * nao);
    const size_t slab = (size_t)S * KC * nchunk * nao;
    __nv_bfloat16* A = reinterpret_cast<__nv_bfloat16*>(p);
    p += al(sizeof(__nv_bfloat16) * slab);
    __nv_bfloat16* B = reinterpret_cast<__nv_bfloat16*>(p);
    p += al(sizeof(__nv_bfloat16) * slab);
    float* C = reinterpret_cast<float*>(p);
    dim3 grid(nchunk, nao);
    k_slice_kernel<S, KC><<<grid, KC, 0, s>>>(X, G, w, nao, ld, npts, nchunk,
                                              ex, ew, A, B);
    OZ_CUDA(cudaGetLastError());
    const float one = 1.0f, zero = 0.0f;
    const long long stride = (long long)S * KC * nao;
    const long long n2 = (long long)nao * nao;
    for (int l = 0; l < S; ++l) {
        OZ_CUBLAS(cublasGemmStridedBatchedEx(
            hb, CUBLAS_OP_T, CUBLAS_OP_N, nao, nao, (l + 1) * KC, &one, A,
            CUDA_R_16BF, S * KC, stride, B + (size_t)(S - 1 - l) * KC,
            CUDA_R_16BF, S * KC, stride, &zero, C + (size_t)l * nchunk * n2,
            CUDA_R_32F, nao, n2, nchunk, CUBLAS_COMPUTE_32F,
            CUBLAS_GEMM_DEFAULT));
    }
    int64_t blocks = (n2 + 255) / 256;
    if (blocks > 152 * 32) blocks = 152 * 32;
    k_combine_kernel<S><<<(unsigned)blocks, 256, 0, s>>>(C, nao, nchunk, ex, ew,
                                                        accumulate, K);
    OZ_CUDA(cudaGetLastError());
    return 0;
}

}  // namespace wb
