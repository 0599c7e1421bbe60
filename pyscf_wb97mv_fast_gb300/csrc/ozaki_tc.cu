// F = fl32(X QD) of the Ozaki split on the fifth-generation tensor cores,
// hand-written: TMA tile loads, tcgen05 MMAs into TMEM, and the exact level
// combination fused into the epilogue (no FP32 level array in HBM).
//
// The split is the one of ozaki.cu (S = 7 balanced 6-bit digits per
// operand, per-point / per-column exponents): the product level l collects
// sum_{i+j=l} A_i B_j over the AO index, every partial sum an integer below
// 2^24, so the FP32 accumulation is exact in any order and the result is
// bitwise the one of the library-GEMM form.
//
// Operand layouts (bf16, K-major, each slice's K extent padded to kp, a
// multiple of 8, and zero beyond nao):
//   A (points x slices x kp):  A[g][i][l] = digit i of X(l, g)
//   B (AOs x slices x kp):     B[mu][j][l] = digit j of QD(l, mu)
// Output tile: 128 points x 64 AOs per CTA.  The seven level accumulators
// live side by side in TMEM (7 x 64 of 512 columns).  For each 64-wide
// block of the AO index the CTA loads the seven B slices (one buffer of
// two) and, one stage at a time, each A slice i; slice i meets B slices
// j = 0 .. 6 - i, four K = 16 MMAs each.  Warp roles: lane 0 of warp 0
// issues the TMA loads, lane 0 of warp 1 the MMAs; all four warps then
// read the accumulators (one TMEM lane per thread), combine the levels in
// int64 and store F.
#include <cuda.h>
#include <cuda_bf16.h>
#include <cudaTypedefs.h>

#include <cstdint>
#include <cstring>
#include <mutex>

#include "launch.hpp"
#include "ozaki.hpp"
#include "ozaki_digits.cuh"
#include "tc_sm100.cuh"

namespace wb {

namespace {

constexpr int S = kOzSlices;
constexpr int kBM = 128;                 // points per tile
constexpr int kBN = 64;                  // AOs per tile
constexpr int kBK = 64;                  // AO index per block (128 B of bf16)
constexpr int kAStages = 4;
constexpr int kATile = kBM * kBK * 2;    // 16 KB
constexpr int kBTile = kBN * kBK * 2;    // 8 KB
constexpr int kBSet = S * kBTile;        // 56 KB: the seven B slices of a block
constexpr int kSmemTiles = 2 * kBSet + kAStages * kATile;
constexpr int kSmemBytes = kSmemTiles + 1024 /* align */ + 256 /* barriers */;
constexpr uint32_t kTmemCols = 512;      // 7 levels x 64 columns
static_assert(S * kBN <= (int)kTmemCols, "levels must fit in TMEM");

__host__ __device__ constexpr int pad8(int n) { return (n + 7) & ~7; }

// -- slicing into the K-major layouts ------------------------------------------

// A: a block per (64 points, 64 AOs); X read along points, A written along
// the AO index (bf16 pairs)
__global__ void __launch_bounds__(256)
f_slice_x_km_kernel(const double* __restrict__ X, int nao, int64_t ld,
                    const int* __restrict__ erow, __nv_bfloat16* __restrict__ A) {
    __shared__ double xs[64][65];
    const int kp = pad8(nao);
    const int64_t g0 = (int64_t)blockIdx.x * 64;
    const int l0 = blockIdx.y * 64;
    const int t = threadIdx.x;
    for (int q = t; q < 64 * 64; q += 256) {
        const int ll = q >> 6, gg = q & 63;
        const int l = l0 + ll;
        const int64_t g = g0 + gg;
        xs[ll][gg] = (l < nao && g < ld) ? X[(int64_t)l * ld + g] : 0.0;
    }
    __syncthreads();
    const int lp = t & 31;                        // AO pair within the block
    const int l = l0 + 2 * lp;
    if (l >= kp) return;
    for (int gg = t >> 5; gg < 64; gg += 8) {
        const int64_t g = g0 + gg;
        if (g >= ld) break;
        const int e = erow[g];
        float d0[S], d1[S];
        digits<S>(xs[2 * lp][gg], e, d0);
        digits<S>(xs[2 * lp + 1][gg], e, d1);
        __nv_bfloat16* row = A + g * (int64_t)S * kp;
#pragma unroll
        for (int i = 0; i < S; ++i)
            *reinterpret_cast<__nv_bfloat162*>(row + (int64_t)i * kp + l) =
                __floats2bfloat162_rn(d0[i], d1[i]);
    }
}

// B: a block per AO column mu of QD (its exponent from the column maximum)
__global__ void __launch_bounds__(256)
f_slice_qd_km_kernel(const double* __restrict__ QD, int nao, int* __restrict__ ecol,
                     __nv_bfloat16* __restrict__ B) {
    const int mu = blockIdx.x;
    const int kp = pad8(nao);
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
    __nv_bfloat16* row = B + (int64_t)mu * S * kp;
    for (int l = threadIdx.x; l < kp; l += blockDim.x) {
        float d[S];
        if (l < nao) {
            digits<S>(QD[(int64_t)l * nao + mu], e, d);
        } else {
#pragma unroll
            for (int i = 0; i < S; ++i) d[i] = 0.0f;
        }
#pragma unroll
        for (int i = 0; i < S; ++i) row[(int64_t)i * kp + l] = __float2bfloat16_rn(d[i]);
    }
}

// -- the GEMM + combine ----------------------------------------------------------

template<typename T>
struct FTcArgs {
    const int* erow;
    const int* ecol;
    T* F;
    int nao;
    int64_t ld;
    int nkb;                      // 64-wide blocks of the AO index
    unsigned long long* status;   // bit 0: a wait gave up
};

template<typename T>
__global__ void __launch_bounds__(128, 1)
ozaki_f_tc_kernel(const __grid_constant__ CUtensorMap mapA,
                  const __grid_constant__ CUtensorMap mapB, const FTcArgs<T> P) {
    extern __shared__ uint8_t smem_raw[];
    const uint32_t raw = tc::smem_u32(smem_raw);
    const uint32_t base = (raw + 1023u) & ~1023u;
    const uint32_t sB = base;                            // 2 x 7 B tiles
    const uint32_t sA = base + 2 * kBSet;                // 4 A stages
    uint8_t* bars_p = smem_raw + (base - raw) + kSmemTiles;
    uint64_t* bars = reinterpret_cast<uint64_t*>(bars_p);
    // barriers: fullB[2], emptyB[2], fullA[4], emptyA[4], done, then the
    // TMEM address slot and the abort flag
    const uint32_t bar0 = tc::smem_u32(bars);
    auto fullB = [&](int b) { return bar0 + 8u * (uint32_t)b; };
    auto emptyB = [&](int b) { return bar0 + 8u * (uint32_t)(2 + b); };
    auto fullA = [&](int s) { return bar0 + 8u * (uint32_t)(4 + s); };
    auto emptyA = [&](int s) { return bar0 + 8u * (uint32_t)(8 + s); };
    const uint32_t done = bar0 + 8u * 12u;
    volatile uint32_t* tslot = reinterpret_cast<volatile uint32_t*>(bars_p + 8 * 13);
    volatile uint32_t* abort_flag = tslot + 1;

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int n0 = blockIdx.x * kBN;
    const int64_t m0 = (int64_t)blockIdx.y * kBM;

    if (threadIdx.x == 0) {
        for (int b = 0; b < 2; ++b) { tc::mbar_init(fullB(b), 1); tc::mbar_init(emptyB(b), 1); }
        for (int s = 0; s < kAStages; ++s) { tc::mbar_init(fullA(s), 1); tc::mbar_init(emptyA(s), 1); }
        tc::mbar_init(done, 1);
        *abort_flag = 0u;
        tc::mbar_init_fence();
        tc::prefetch_map(&mapA);
        tc::prefetch_map(&mapB);
    }
    if (warp == 0) tc::tmem_alloc(tc::smem_u32((const void*)tslot), kTmemCols);
    tc::tc_fence_before();
    __syncthreads();
    tc::tc_fence_after();
    const uint32_t tmem = *tslot;
    const int nkb = P.nkb;

    // loads issued per A stage / B buffer (the producer's count; the last
    // one's phase is what the clean-up waits for)
    int issuedA[kAStages] = {0, 0, 0, 0}, issuedB[2] = {0, 0};
    if (warp == 0 && lane == 0) {
        // producer: per AO block the seven B slices, then A slice by slice
        int it = 0;
        for (int kb = 0; kb < nkb && !*abort_flag; ++kb) {
            const int bs = kb & 1;
            if (kb >= 2 && !tc::mbar_wait(emptyB(bs), ((kb >> 1) - 1) & 1)) {
                *abort_flag = 1u;
                break;
            }
            tc::mbar_expect_tx(fullB(bs), kBSet);
            ++issuedB[bs];
            for (int j = 0; j < S; ++j)
                tc::tma_load_3d(sB + bs * kBSet + j * kBTile, &mapB, kb * kBK, j, n0,
                                fullB(bs));
            for (int i = 0; i < S; ++i, ++it) {
                const int s = it % kAStages;
                if (it >= kAStages &&
                    !tc::mbar_wait(emptyA(s), ((it / kAStages) - 1) & 1)) {
                    *abort_flag = 1u;
                    break;
                }
                tc::mbar_expect_tx(fullA(s), kATile);
                ++issuedA[s];
                tc::tma_load_3d(sA + s * kATile, &mapA, kb * kBK, i, (int)m0, fullA(s));
            }
        }
    } else if (warp == 1 && lane == 0) {
        // MMA issue: level i + j accumulates A_i B_j
        constexpr uint32_t idesc = tc::idesc_bf16_f32<kBM, kBN>();
        int it = 0;
        bool ok = true;
        for (int kb = 0; kb < nkb && ok; ++kb) {
            const int bs = kb & 1;
            if (!tc::mbar_wait(fullB(bs), (kb >> 1) & 1)) { ok = false; break; }
            for (int i = 0; i < S; ++i, ++it) {
                const int s = it % kAStages;
                if (!tc::mbar_wait(fullA(s), (it / kAStages) & 1)) { ok = false; break; }
                tc::tc_fence_after();
                const uint32_t a_addr = sA + s * kATile;
                for (int j = 0; j + i < S; ++j) {
                    const uint32_t b_addr = sB + bs * kBSet + j * kBTile;
                    const uint32_t d = tmem + (uint32_t)((i + j) * kBN);
#pragma unroll
                    for (int k = 0; k < kBK / 16; ++k) {
                        const uint64_t ad = tc::desc_kmajor_sw128(a_addr + 32u * k);
                        const uint64_t bd = tc::desc_kmajor_sw128(b_addr + 32u * k);
                        tc::mma_bf16(d, ad, bd, idesc,
                                     (kb > 0 || i > 0 || k > 0) ? 1u : 0u);
                    }
                }
                tc::mma_commit(emptyA(s));
            }
            if (!ok) break;
            tc::mma_commit(emptyB(bs));
        }
        if (!ok) *abort_flag = 1u;
        tc::mma_commit(done);
    }
    __syncwarp();

    // epilogue: every thread owns one point (TMEM lane) of the tile
    const bool ok_done = tc::mbar_wait(done, 0);
    tc::tc_fence_after();
    const bool bad = !ok_done || *abort_flag;
    const int64_t g = m0 + 32 * warp + lane;
    const int er = g < P.ld ? P.erow[g] : 0;
    const uint32_t tl = tmem + ((uint32_t)(32 * warp) << 16);
#pragma unroll 1
    for (int c = 0; c < kBN / 16; ++c) {
        long long acc[16];
#pragma unroll
        for (int q = 0; q < 16; ++q) acc[q] = 0;
#pragma unroll
        for (int l = 0; l < S; ++l) {
            float v[16];
            tc::tmem_ld16(tl + (uint32_t)(l * kBN + 16 * c), v);
#pragma unroll
            for (int q = 0; q < 16; ++q)
                acc[q] += ((long long)__float2int_rn(v[q])) << (kB * (S - 1 - l));
        }
        if (g < P.ld) {
#pragma unroll
            for (int q = 0; q < 16; ++q) {
                const int mu = n0 + 16 * c + q;
                if (mu < P.nao) {
                    const int sc = er + P.ecol[mu] - 2 * kW + 2 + kB * (S - 1);
                    P.F[(int64_t)mu * P.ld + g] =
                        bad ? (T)__int_as_float(0x7fc00000) : scaled_ll_to<T>(acc[q], sc);
                }
            }
        }
    }
    if (bad && threadIdx.x == 0) atomicOr(P.status, 1ull);
    tc::tc_fence_before();
    __syncthreads();
    if (threadIdx.x == 0) {
        // every TMA load this CTA issued has landed before the CTA exits (at
        // once on the normal path, where the MMAs consumed them all)
        for (int st = 0; st < kAStages; ++st)
            if (issuedA[st]) tc::mbar_wait(fullA(st), (issuedA[st] - 1) & 1);
        for (int b = 0; b < 2; ++b)
            if (issuedB[b]) tc::mbar_wait(fullB(b), (issuedB[b] - 1) & 1);
    }
    __syncthreads();
    if (warp == 0) tc::tmem_dealloc(tmem, kTmemCols);
}

// -- host: tensor maps -------------------------------------------------------------

PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000,
                                             cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
    });
    return fn;
}

// (rows x S slices x kp) bf16, K-major, box 64 (K) x 1 x box_rows, 128-byte
// swizzle, zero fill beyond nao along K and beyond rows
bool make_map(CUtensorMap* m, const void* base, int nao, int64_t rows, int box_rows) {
    auto fn = encode_fn();
    if (!fn) return false;
    const int kp = pad8(nao);
    cuuint64_t dims[3] = {(cuuint64_t)nao, (cuuint64_t)S, (cuuint64_t)rows};
    cuuint64_t strides[2] = {(cuuint64_t)kp * 2, (cuuint64_t)S * kp * 2};
    cuuint32_t box[3] = {(cuuint32_t)kBK, 1u, (cuuint32_t)box_rows};
    cuuint32_t estr[3] = {1u, 1u, 1u};
    return fn(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 3, const_cast<void*>(base), dims,
              strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
              CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
              CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

inline size_t al(size_t x) { return (x + 255) & ~(size_t)255; }

}  // namespace

size_t ozaki_f_tc_bytes(int nao, int64_t ld) {
    const size_t kp = (size_t)pad8(nao);
    return al(sizeof(int) * ld) + al(sizeof(int) * nao) +
           al(sizeof(__nv_bfloat16) * (size_t)ld * S * kp) +
           al(sizeof(__nv_bfloat16) * (size_t)nao * S * kp) +
           al(sizeof(unsigned long long));
}

template<typename T>
static int f_gemm_tc_t(const double* X, const double* QD, int nao, int64_t ld, T* F,
                       void* ws, cudaStream_t s, unsigned long long* status) {
    if (!ozaki_f_supported(nao) || ld % 2 != 0 || ld > (int64_t)kBM * 65535)
        return (int)cudaErrorInvalidValue;
    const size_t kp = (size_t)pad8(nao);
    char* p = static_cast<char*>(ws);
    int* erow = reinterpret_cast<int*>(p); p += al(sizeof(int) * ld);
    int* ecol = reinterpret_cast<int*>(p); p += al(sizeof(int) * nao);
    __nv_bfloat16* A = reinterpret_cast<__nv_bfloat16*>(p);
    p += al(sizeof(__nv_bfloat16) * (size_t)ld * S * kp);
    __nv_bfloat16* B = reinterpret_cast<__nv_bfloat16*>(p);
    p += al(sizeof(__nv_bfloat16) * (size_t)nao * S * kp);
    if (!status) status = reinterpret_cast<unsigned long long*>(p);

    CUtensorMap mapA, mapB;
    if (!make_map(&mapA, A, nao, ld, kBM) || !make_map(&mapB, B, nao, nao, kBN))
        return (int)cudaErrorNotSupported;
    cudaError_t e = cudaFuncSetAttribute(ozaki_f_tc_kernel<T>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         kSmemBytes);
    if (e != cudaSuccess) return (int)e;
    f_rowmax(X, nao, ld, erow, s);
    {
        dim3 grid((unsigned)((ld + 63) / 64), (unsigned)((kp + 63) / 64));
        f_slice_x_km_kernel<<<grid, 256, 0, s>>>(X, nao, ld, erow, A);
    }
    f_slice_qd_km_kernel<<<nao, 256, 0, s>>>(QD, nao, ecol, B);
    FTcArgs<T> a{erow, ecol, F, nao, ld, (nao + kBK - 1) / kBK, status};
    dim3 grid((unsigned)((nao + kBN - 1) / kBN), (unsigned)((ld + kBM - 1) / kBM));
    ozaki_f_tc_kernel<T><<<grid, 128, kSmemBytes, s>>>(mapA, mapB, a);
    return (int)cudaGetLastError();
}

int ozaki_f_gemm_tc(const double* X, const double* QD, int nao, int64_t ld, float* F,
                    void* ws, cudaStream_t s, unsigned long long* status) {
    return f_gemm_tc_t<float>(X, QD, nao, ld, F, ws, s, status);
}

int ozaki_f_gemm_tc64(const double* X, const double* QD, int nao, int64_t ld, double* F,
                      void* ws, cudaStream_t s, unsigned long long* status) {
    return f_gemm_tc_t<double>(X, QD, nao, ld, F, ws, s, status);
}

}  // namespace wb
