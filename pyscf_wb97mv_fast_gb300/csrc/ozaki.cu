// FP64-accurate GEMMs of the COSX K build on the bf16 tensor cores.
//
// GB300 runs FP64 at ~1 TFLOP/s, so F = X QD and K = X^T (w o G) -- the
// two dense contractions the reference keeps in FP64 (gpu/sgx_k.py:14-28,
// :722, :734) -- would dominate the build.  They run here as an Ozaki
// split (K. Ozaki et al., Numer. Algorithms 59 (2012) 95-118; on tensor
// cores: H. Ootomo, K. Ozaki, R. Yokota, IJHPCA 2024):
//
//   x = 2^(e-W+1) sum_i d_i 2^(B (S-1-i)),  |d_i| <= 2^(B-1)  (bf16-exact)
//
// with e per row / column (chunk), B = 6-bit balanced digits, S = 7 slices
// (W = 42 bits), the digits cut from rint(x 2^(W-1-e)) with integer ops.
// A product level l = i + j collects sum_{i+j=l} A_i B_j in ONE bf16 GEMM
// with FP32 accumulation: storing the A slices ascending and the B slices
// descending along K makes every level a prefix of A times a suffix of B.
// Every product is an integer of magnitude <= 2^(2B-2) = 1024 and a level
// sums at most (l+1) * Kc of them, so with (l+1) Kc < 2^14 every partial
// sum is an integer below 2^24: the FP32 accumulation is exact, whatever
// order the tensor cores use.  Levels are combined exactly in int64 and
// scaled once in FP64.  The result carries W = 42 bits relative to the
// per-row / per-column maxima; the truncated products (i + j >= S) are
// below 2^-W of them.
//
// The level GEMMs are library GEMMs by default (cuBLAS bf16 GEMMs with FP32
// accumulation, one per level) around this file's slicing and combination
// kernels.  ozaki_set_f_engine(kOzEngineTc) runs the F product on this
// library's own tensor-core kernel instead (ozaki_tc.cu: TMA, tcgen05 MMAs
// into TMEM, the level combination fused into its epilogue) -- bitwise the
// same result; its seven exact level accumulators leave room for 64-wide
// N tiles only, and it measured 2.4x slower than the library form on the
// bench step (18.4 vs 7.65 ms).  The K product's level GEMMs are cuBLAS.
#include <cublas_v2.h>
#include <cuda_bf16.h>

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdint>

#include "launch.hpp"
#include "ozaki.hpp"
#include "ozaki_digits.cuh"

namespace wb {

// ---------------------------------------------------------------------------
// F = X QD.  X (nao, ld) AO-major = column-major A (ld x nao) scaled per row
// g; QD row-major = column-major Q (nao x nao) with Q(mu, l) = QD(l, mu);
// B = Q^T scaled per column mu (= per row mu of Q).
// A_all (ld x S*nao, col-major): column block i = slice i.
// B_all (S*nao x nao, col-major): row block r = slice S-1-r.
// ---------------------------------------------------------------------------
// exponent of max_l |X(l, g)| per point g: eight rows in flight per thread
__global__ void f_rowmax_kernel(const double* __restrict__ X, int nao,
                                int64_t ld, int* __restrict__ erow) {
    const int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= ld) return;
    const unsigned long long* Xb = reinterpret_cast<const unsigned long long*>(X);
    unsigned long long m = 0;
    int l = 0;
    for (; l + 8 <= nao; l += 8) {
        unsigned long long b[8];
#pragma unroll
        for (int u = 0; u < 8; ++u) b[u] = __ldg(Xb + (int64_t)(l + u) * ld + g);
#pragma unroll
        for (int u = 0; u < 8; ++u) {
            const unsigned long long a = b[u] & 0x7fffffffffffffffull;
            m = a > m ? a : m;
        }
    }
    for (; l < nao; ++l) {
        const unsigned long long a = __ldg(Xb + (int64_t)l * ld + g) & 0x7fffffffffffffffull;
        m = a > m ? a : m;
    }
    erow[g] = exp_of_bits(m);
}

// slices of X: one thread per (row l, two points); bf16 pairs per store
template<int S>
__global__ void f_slice_x_kernel(const double* __restrict__ X, int nao,
                                 int64_t ld, const int* __restrict__ erow,
                                 __nv_bfloat16* __restrict__ A) {
    const int l = blockIdx.y;
    const int64_t g = 2 * ((int64_t)blockIdx.x * blockDim.x + threadIdx.x);
    if (g >= ld) return;                    // ld is even (a multiple of 32)
    const double2 x = *reinterpret_cast<const double2*>(X + (int64_t)l * ld + g);
    const int2 e = *reinterpret_cast<const int2*>(erow + g);
    float d0[S], d1[S];
    digits<S>(x.x, e.x, d0);
    digits<S>(x.y, e.y, d1);
#pragma unroll
    for (int i = 0; i < S; ++i)
        *reinterpret_cast<__nv_bfloat162*>(A + ((int64_t)i * nao + l) * ld + g) =
            __floats2bfloat162_rn(d0[i], d1[i]);
}

template<int S>
__global__ void f_slice_qd_kernel(const double* __restrict__ QD, int nao,
                                  int* __restrict__ ecol,
                                  __nv_bfloat16* __restrict__ B) {
    // one block per column mu of B = Q^T, i.e. QD(:, mu)
    const int mu = blockIdx.x;
    __shared__ unsigned long long red[256];
    unsigned long long m = 0;
    for (int l = threadIdx.x; l < nao; l += blockDim.x) {
        const unsigned long long b =
            (unsigned long long)__double_as_longlong(QD[(int64_t)l * nao + mu]) &
            0x7fffffffffffffffull;
        m = b > m ? b : m;
    }
    red[threadIdx.x] = m;
    __syncthreads();
    for (int s = blockDim.x / 2; s > 0; s >>= 1) {
        if (threadIdx.x < s && red[threadIdx.x + s] > red[threadIdx.x])
            red[threadIdx.x] = red[threadIdx.x + s];
        __syncthreads();
    }
    const int e = exp_of_bits(red[0]);
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

// x y = 2^(e+f-2W+2) sum_l C_l 2^(B (2S-2-l))
//     = 2^(e+f-2W+2+B(S-1)) * [sum_l C_l 2^(B (S-1-l))]
template<int S, typename T>
__global__ void f_combine_kernel(const float* __restrict__ C, int nao,
                                 int64_t ld, const int* __restrict__ erow,
                                 const int* __restrict__ ecol,
                                 T* __restrict__ F) {
    const int mu = blockIdx.y;
    const int64_t g = 4 * ((int64_t)blockIdx.x * blockDim.x + threadIdx.x);
    if (g >= ld) return;                    // ld is a multiple of 4
    const int64_t plane = (int64_t)nao * ld;
    const int64_t i = (int64_t)mu * ld + g;
    float4 c[S];
#pragma unroll
    for (int l = 0; l < S; ++l)
        c[l] = __ldg(reinterpret_cast<const float4*>(C + (int64_t)l * plane + i));
    const int4 er = *reinterpret_cast<const int4*>(erow + g);
    const int base = ecol[mu] - 2 * kW + 2 + kB * (S - 1);
    float v[4][S];
#pragma unroll
    for (int l = 0; l < S; ++l) {
        v[0][l] = c[l].x; v[1][l] = c[l].y; v[2][l] = c[l].z; v[3][l] = c[l].w;
    }
    const T o0 = scaled_ll_to<T>(combine_levels<S>(v[0]), er.x + base);
    const T o1 = scaled_ll_to<T>(combine_levels<S>(v[1]), er.y + base);
    const T o2 = scaled_ll_to<T>(combine_levels<S>(v[2]), er.z + base);
    const T o3 = scaled_ll_to<T>(combine_levels<S>(v[3]), er.w + base);
    if constexpr (sizeof(T) == 4) {
        *reinterpret_cast<float4*>(F + i) = make_float4(o0, o1, o2, o3);
    } else {
        *reinterpret_cast<double2*>(F + i) = make_double2(o0, o1);
        *reinterpret_cast<double2*>(F + i + 2) = make_double2(o2, o3);
    }
}

// ---------------------------------------------------------------------------
// K = X^T (w o G), K dimension = grid points, chunked by KC points with a
// scale per (chunk, column).  Per chunk c, A_c(k, mu) = X[mu, c KC + k] and
// B_c(k, nu) = w_k G[nu, c KC + k]; layouts (col-major, ld = S KC):
//   A: column mu = [slice 0 (KC) | slice 1 | ... ]     (ascending)
//   B: column nu = [slice S-1 | ... | slice 0]          (descending)
// chunk stride S KC nao.  One CTA of 256 threads per (chunk, column).
// ---------------------------------------------------------------------------
// DOX = false: the X slices and exponents of this tile are already in A /
// ex (an earlier omega of the same tile); only w o G is sliced.  B holds nb
// columns per chunk (several right-hand sides side by side); this launch
// fills columns boff .. boff + nao - 1.
template<int S, int KC, bool DOX, typename GT>
__global__ void __launch_bounds__(KC / 8, 4)
k_slice_kernel(const double* __restrict__ X, const GT* __restrict__ G,
               const double* __restrict__ w, int nao, int64_t ld,
               int64_t npts, int* __restrict__ ex, int* __restrict__ ew,
               __nv_bfloat16* __restrict__ A, __nv_bfloat16* __restrict__ B,
               int nb, int boff) {
    constexpr int T = KC / 8;               // threads: eight points each
    const int c = blockIdx.x, col = blockIdx.y;
    __shared__ unsigned long long rx[T / 32], rw[T / 32];
    const int k0 = 8 * threadIdx.x;
    const int64_t g0 = (int64_t)c * KC + k0;
    double xv[8], wv[8];
    unsigned long long mx = 0, mw = 0;
    if (g0 + 8 <= npts) {
        const double2* xp = reinterpret_cast<const double2*>(X + (int64_t)col * ld + g0);
        const double2* wp = reinterpret_cast<const double2*>(w + g0);
        double gv[8];
        if constexpr (sizeof(GT) == 4) {
            const float4* gp = reinterpret_cast<const float4*>(G + (int64_t)col * ld + g0);
            const float4 ga = __ldg(gp), gb = __ldg(gp + 1);
            gv[0] = ga.x; gv[1] = ga.y; gv[2] = ga.z; gv[3] = ga.w;
            gv[4] = gb.x; gv[5] = gb.y; gv[6] = gb.z; gv[7] = gb.w;
        } else {
            const double2* gp = reinterpret_cast<const double2*>(G + (int64_t)col * ld + g0);
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                const double2 t = __ldg(gp + u);
                gv[2 * u] = t.x;
                gv[2 * u + 1] = t.y;
            }
        }
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            const double2 b = __ldg(wp + u);
            if (DOX) {
                const double2 a = __ldg(xp + u);
                xv[2 * u] = a.x; xv[2 * u + 1] = a.y;
            } else {
                xv[2 * u] = 0.0; xv[2 * u + 1] = 0.0;
            }
            wv[2 * u] = b.x * gv[2 * u];
            wv[2 * u + 1] = b.y * gv[2 * u + 1];
        }
    } else {
#pragma unroll
        for (int u = 0; u < 8; ++u) {
            const int64_t g = g0 + u;
            xv[u] = 0.0;
            wv[u] = 0.0;
            if (g < npts) {
                if (DOX) xv[u] = X[(int64_t)col * ld + g];
                wv[u] = w[g] * (double)G[(int64_t)col * ld + g];
            }
        }
    }
#pragma unroll
    for (int u = 0; u < 8; ++u) {
        const unsigned long long bx =
            (unsigned long long)__double_as_longlong(xv[u]) & 0x7fffffffffffffffull;
        const unsigned long long bw =
            (unsigned long long)__double_as_longlong(wv[u]) & 0x7fffffffffffffffull;
        mx = bx > mx ? bx : mx;
        mw = bw > mw ? bw : mw;
    }
    for (int o = 16; o > 0; o >>= 1) {
        const unsigned long long ox = __shfl_xor_sync(0xffffffffu, mx, o);
        const unsigned long long ow = __shfl_xor_sync(0xffffffffu, mw, o);
        mx = ox > mx ? ox : mx;
        mw = ow > mw ? ow : mw;
    }
    const int warp = threadIdx.x >> 5;
    if ((threadIdx.x & 31) == 0) { rx[warp] = mx; rw[warp] = mw; }
    __syncthreads();
    mx = 0;
    mw = 0;
#pragma unroll
    for (int j = 0; j < T / 32; ++j) {
        mx = rx[j] > mx ? rx[j] : mx;
        mw = rw[j] > mw ? rw[j] : mw;
    }
    const int e1 = exp_of_bits(mx), e2 = exp_of_bits(mw);
    if (threadIdx.x == 0) {
        if (DOX) ex[(int64_t)c * nao + col] = e1;
        ew[(int64_t)c * nb + boff + col] = e2;
    }
    const int64_t colbase = (int64_t)c * S * KC * nao + (int64_t)col * S * KC;
    const int64_t colbase_b = (int64_t)c * S * KC * nb + (int64_t)(boff + col) * S * KC;
    // one operand's digits at a time: the X slices, then the w o G ones
    // (half the live registers of both at once)
    auto store = [&](const double* v, const int e, __nv_bfloat16* dst, const bool desc) {
        float d[8][S];
#pragma unroll
        for (int u = 0; u < 8; ++u) digits<S>(v[u], e, d[u]);
#pragma unroll
        for (int i = 0; i < S; ++i) {
            __nv_bfloat162 p[4];
#pragma unroll
            for (int u = 0; u < 4; ++u)
                p[u] = __floats2bfloat162_rn(d[2 * u][i], d[2 * u + 1][i]);
            *reinterpret_cast<uint4*>(dst + (int64_t)(desc ? S - 1 - i : i) * KC + k0) =
                *reinterpret_cast<const uint4*>(p);
        }
    };
    if (DOX) store(xv, e1, A + colbase, false);
    store(wv, e2, B + colbase_b, true);
}

// K_r[mu, nu] (+)= sum_c 2^(ex+ew-2W+2+B(S-1)) [sum_l C[l][c] 2^(B (S-1-l))]
// for the nb / nao right-hand sides r (column r nao + nu of C)
struct KOut {
    double* k[8];
};

template<int S>
__global__ void k_combine_kernel(const float* __restrict__ C, int nao, int nb,
                                 int nchunk, const int* __restrict__ ex,
                                 const int* __restrict__ ew, int accumulate,
                                 const KOut Ks) {
    const int64_t nc = (int64_t)nao * nb;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < nc;
         i += (int64_t)gridDim.x * blockDim.x) {
        const int mu = (int)(i % nao), col = (int)(i / nao);   // C col-major
        double acc = 0.0;
        // four chunks' loads in flight at once; the sum stays in chunk order
        constexpr int U = 4;
        int c = 0;
        for (; c + U <= nchunk; c += U) {
            float v[U][S];
            int sc[U];
#pragma unroll
            for (int u = 0; u < U; ++u) {
#pragma unroll
                for (int l = 0; l < S; ++l)
                    v[u][l] = __ldg(C + ((int64_t)l * nchunk + c + u) * nc + i);
                sc[u] = ex[(int64_t)(c + u) * nao + mu] + ew[(int64_t)(c + u) * nb + col] -
                        2 * kW + 2 + kB * (S - 1);
            }
#pragma unroll
            for (int u = 0; u < U; ++u) acc += (double)combine_levels<S>(v[u]) * pow2(sc[u]);
        }
        for (; c < nchunk; ++c) {
            float v[S];
#pragma unroll
            for (int l = 0; l < S; ++l) v[l] = C[((int64_t)l * nchunk + c) * nc + i];
            const long long lv = combine_levels<S>(v);
            const int sc = ex[(int64_t)c * nao + mu] + ew[(int64_t)c * nb + col] -
                           2 * kW + 2 + kB * (S - 1);
            acc += (double)lv * pow2(sc);
        }
        double* K = Ks.k[col / nao];
        const int64_t o = (int64_t)mu * nao + col % nao;       // K row-major
        K[o] = accumulate ? K[o] + acc : acc;
    }
}

// ---------------------------------------------------------------------------
static inline size_t al(size_t x) { return (x + 255) & ~(size_t)255; }

size_t ozaki_f_bytes(int nao, int64_t ld) {
    const size_t S = kOzSlices;
    const size_t lib = al(sizeof(int) * ld) + al(sizeof(int) * nao) +
                       al(sizeof(__nv_bfloat16) * S * nao * ld) +
                       al(sizeof(__nv_bfloat16) * S * nao * nao) +
                       al(sizeof(float) * S * nao * ld);
    return std::max(lib, ozaki_f_tc_bytes(nao, ld));
}

size_t ozaki_k_bytes(int nao, int64_t ld, int nrhs) {
    const size_t S = kOzSlices;
    const int64_t nchunk = (ld + kOzKc - 1) / kOzKc;
    return al(sizeof(int) * nchunk * nao) + al(sizeof(int) * nchunk * nao * nrhs) +
           al(sizeof(__nv_bfloat16) * S * kOzKc * nchunk * nao) +
           al(sizeof(__nv_bfloat16) * S * kOzKc * nchunk * nao * nrhs) +
           al(sizeof(float) * S * nchunk * (size_t)nao * nao * nrhs);
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

void f_rowmax(const double* X, int nao, int64_t ld, int* erow, cudaStream_t s) {
    f_rowmax_kernel<<<(unsigned)((ld + 255) / 256), 256, 0, s>>>(X, nao, ld, erow);
}

namespace {
std::atomic<int> g_f_engine{kOzEngineLibrary};
}

void ozaki_set_f_engine(int engine) { g_f_engine.store(engine); }
int ozaki_get_f_engine() { return g_f_engine.load(); }

int ozaki_f_gemm(cublasHandle_t hb, const double* X, const double* QD,
                 int nao, int64_t ld, float* F, void* ws, cudaStream_t s,
                 unsigned long long* status) {
    if (g_f_engine.load() == kOzEngineTc)
        return ozaki_f_gemm_tc(X, QD, nao, ld, F, ws, s, status);
    return ozaki_f_gemm_cublas(hb, X, QD, nao, ld, F, ws, s);
}

int ozaki_f_gemm64(cublasHandle_t hb, const double* X, const double* QD,
                   int nao, int64_t ld, double* F, void* ws, cudaStream_t s,
                   unsigned long long* status) {
    if (g_f_engine.load() == kOzEngineTc)
        return ozaki_f_gemm_tc64(X, QD, nao, ld, F, ws, s, status);
    return ozaki_f_gemm_cublas64(hb, X, QD, nao, ld, F, ws, s);
}

template<typename T>
static int f_gemm_cublas_t(cublasHandle_t hb, const double* X, const double* QD,
                           int nao, int64_t ld, T* F, void* ws, cudaStream_t s) {
    constexpr int S = kOzSlices;
    char* p = static_cast<char*>(ws);
    int* erow = reinterpret_cast<int*>(p); p += al(sizeof(int) * ld);
    int* ecol = reinterpret_cast<int*>(p); p += al(sizeof(int) * nao);
    __nv_bfloat16* A = reinterpret_cast<__nv_bfloat16*>(p);
    p += al(sizeof(__nv_bfloat16) * (size_t)S * nao * ld);
    __nv_bfloat16* B = reinterpret_cast<__nv_bfloat16*>(p);
    p += al(sizeof(__nv_bfloat16) * (size_t)S * nao * nao);
    float* C = reinterpret_cast<float*>(p);
    f_rowmax_kernel<<<(unsigned)((ld + 255) / 256), 256, 0, s>>>(X, nao, ld, erow);
    OZ_CUDA(cudaGetLastError());
    {
        dim3 grid((unsigned)((ld / 2 + 255) / 256), (unsigned)nao);
        f_slice_x_kernel<S><<<grid, 256, 0, s>>>(X, nao, ld, erow, A);
        OZ_CUDA(cudaGetLastError());
    }
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
    {
        dim3 grid((unsigned)((ld / 4 + 255) / 256), (unsigned)nao);
        f_combine_kernel<S, T><<<grid, 256, 0, s>>>(C, nao, ld, erow, ecol, F);
        OZ_CUDA(cudaGetLastError());
    }
    return 0;
}

int ozaki_f_gemm_cublas(cublasHandle_t hb, const double* X, const double* QD,
                        int nao, int64_t ld, float* F, void* ws, cudaStream_t s) {
    return f_gemm_cublas_t<float>(hb, X, QD, nao, ld, F, ws, s);
}

int ozaki_f_gemm_cublas64(cublasHandle_t hb, const double* X, const double* QD,
                          int nao, int64_t ld, double* F, void* ws, cudaStream_t s) {
    return f_gemm_cublas_t<double>(hb, X, QD, nao, ld, F, ws, s);
}

template<typename GT>
static int k_gemm_multi_t(cublasHandle_t hb, const double* X, const GT* const* G,
                          int nrhs, const double* w, int nao, int64_t ld,
                          int64_t npts, int accumulate, double* const* K, void* ws,
                          cudaStream_t s, bool x_sliced) {
    constexpr int S = kOzSlices, KC = kOzKc;
    if (nrhs < 1 || nrhs > 8) return (int)cudaErrorInvalidValue;
    const int nchunk = (int)((ld + KC - 1) / KC);
    const int nb = nrhs * nao;
    // the X side (ex, A) first, at offsets independent of nrhs, so that a
    // later call with x_sliced finds them whatever its nrhs
    char* p = static_cast<char*>(ws);
    int* ex = reinterpret_cast<int*>(p); p += al(sizeof(int) * (size_t)nchunk * nao);
    const size_t slab = (size_t)S * KC * nchunk * nao;
    __nv_bfloat16* A = reinterpret_cast<__nv_bfloat16*>(p);
    p += al(sizeof(__nv_bfloat16) * slab);
    int* ew = reinterpret_cast<int*>(p); p += al(sizeof(int) * (size_t)nchunk * nb);
    __nv_bfloat16* B = reinterpret_cast<__nv_bfloat16*>(p);
    p += al(sizeof(__nv_bfloat16) * slab * nrhs);
    float* C = reinterpret_cast<float*>(p);
    KOut Kd = {};
    for (int r = 0; r < nrhs; ++r) Kd.k[r] = K[r];
    dim3 grid(nchunk, nao);
    for (int r = 0; r < nrhs; ++r) {
        if (x_sliced || r > 0)
            k_slice_kernel<S, KC, false, GT><<<grid, KC / 8, 0, s>>>(
                X, G[r], w, nao, ld, npts, ex, ew, A, B, nb, r * nao);
        else
            k_slice_kernel<S, KC, true, GT><<<grid, KC / 8, 0, s>>>(
                X, G[r], w, nao, ld, npts, ex, ew, A, B, nb, r * nao);
        OZ_CUDA(cudaGetLastError());
    }
    const float one = 1.0f, zero = 0.0f;
    const long long stride_a = (long long)S * KC * nao;
    const long long stride_b = (long long)S * KC * nb;
    const long long nc = (long long)nao * nb;
    for (int l = 0; l < S; ++l) {
        OZ_CUBLAS(cublasGemmStridedBatchedEx(
            hb, CUBLAS_OP_T, CUBLAS_OP_N, nao, nb, (l + 1) * KC, &one, A,
            CUDA_R_16BF, S * KC, stride_a, B + (size_t)(S - 1 - l) * KC,
            CUDA_R_16BF, S * KC, stride_b, &zero, C + (size_t)l * nchunk * nc,
            CUDA_R_32F, nao, nc, nchunk, CUBLAS_COMPUTE_32F,
            CUBLAS_GEMM_DEFAULT));
    }
    const int64_t blocks = grid_stride_blocks(nc, 256, 32);
    k_combine_kernel<S><<<(unsigned)blocks, 256, 0, s>>>(C, nao, nb, nchunk, ex, ew,
                                                        accumulate, Kd);
    OZ_CUDA(cudaGetLastError());
    return 0;
}

int ozaki_k_gemm_multi(cublasHandle_t hb, const double* X, const float* const* G,
                       int nrhs, const double* w, int nao, int64_t ld,
                       int64_t npts, int accumulate, double* const* K, void* ws,
                       cudaStream_t s, bool x_sliced) {
    return k_gemm_multi_t<float>(hb, X, G, nrhs, w, nao, ld, npts, accumulate, K, ws, s,
                                 x_sliced);
}

int ozaki_k_gemm64(cublasHandle_t hb, const double* X, const double* G,
                   const double* w, int nao, int64_t ld, int64_t npts,
                   int accumulate, double* K, void* ws, cudaStream_t s) {
    return k_gemm_multi_t<double>(hb, X, &G, 1, w, nao, ld, npts, accumulate, &K, ws, s,
                                  false);
}

int ozaki_k_gemm(cublasHandle_t hb, const double* X, const float* G,
                 const double* w, int nao, int64_t ld, int64_t npts,
                 int accumulate, double* K, void* ws, cudaStream_t s,
                 bool x_sliced) {
    return ozaki_k_gemm_multi(hb, X, &G, 1, w, nao, ld, npts, accumulate, &K, ws,
                              s, x_sliced);
}

}  // namespace wb
