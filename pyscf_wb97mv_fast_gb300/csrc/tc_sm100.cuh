// Blackwell (sm_100 family) building blocks in inline PTX: mbarriers with
// bounded waits, TMA tiled tensor loads, and the fifth-generation tensor
// core (tcgen05: TMEM allocation, MMA issue, commit, TMEM loads) with its
// shared-memory and instruction descriptors.
//
// Every wait polls a bounded number of times; a wait that gives up sets a
// flag (the caller reports it to the host) instead of spinning forever.
#pragma once
#include <cuda.h>
#include <cuda_runtime.h>

#include <cstdint>

namespace wb {
namespace tc {

// polls before a wait gives up (about a second of polling at the least)
constexpr unsigned kSpinLimit = 1u << 26;

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}

// -- mbarriers ---------------------------------------------------------------
__device__ __forceinline__ void mbar_init(const uint32_t bar, const uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" :: "r"(bar), "r"(count)
                 : "memory");
}
__device__ __forceinline__ void mbar_init_fence() {
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
}
__device__ __forceinline__ void mbar_expect_tx(const uint32_t bar, const uint32_t bytes) {
    asm volatile("{\n\t.reg .b64 st;\n\t"
                 "mbarrier.arrive.expect_tx.shared::cta.b64 st, [%0], %1;\n\t}\n"
                 :: "r"(bar), "r"(bytes) : "memory");
}
// true once the phase with the given parity has completed; false when the
// poll limit ran out
__device__ __forceinline__ bool mbar_wait(const uint32_t bar, const uint32_t parity) {
    for (unsigned i = 0; i < kSpinLimit; ++i) {
        uint32_t ok;
        asm volatile("{\n\t.reg .pred p;\n\t"
                     "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
                     "selp.u32 %0, 1, 0, p;\n\t}\n"
                     : "=r"(ok) : "r"(bar), "r"(parity) : "memory");
        if (ok) return true;
    }
    return false;
}

// -- TMA ---------------------------------------------------------------------
// 3-D tiled load of the box at (c0, c1, c2) (c0 innermost, in elements)
// into shared memory; completes on bar (complete_tx)
__device__ __forceinline__ void tma_load_3d(const uint32_t dst, const CUtensorMap* map,
                                            const int c0, const int c1, const int c2,
                                            const uint32_t bar) {
    asm volatile("cp.async.bulk.tensor.3d.shared::cluster.global.tile"
                 ".mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], [%5];\n"
                 :: "r"(dst), "l"(reinterpret_cast<uint64_t>(map)), "r"(c0), "r"(c1),
                    "r"(c2), "r"(bar)
                 : "memory");
}
__device__ __forceinline__ void prefetch_map(const CUtensorMap* map) {
    asm volatile("prefetch.tensormap [%0];\n" :: "l"(reinterpret_cast<uint64_t>(map))
                 : "memory");
}

// -- tcgen05 -------------------------------------------------------------------
// warp-wide: allocate ncols TMEM columns (a power of two >= 32); the TMEM
// address is written to the shared-memory word at slot
__device__ __forceinline__ void tmem_alloc(const uint32_t slot, const uint32_t ncols) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n"
                 :: "r"(slot), "r"(ncols) : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n"
                 ::: "memory");
}
__device__ __forceinline__ void tmem_dealloc(const uint32_t taddr, const uint32_t ncols) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n"
                 :: "r"(taddr), "r"(ncols) : "memory");
}
__device__ __forceinline__ void tc_fence_before() {
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
}
__device__ __forceinline__ void tc_fence_after() {
    asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
}

// D[tmem] (+)= A[smem] B[smem]^T, one thread issues; accumulate = 0
// overwrites D
__device__ __forceinline__ void mma_bf16(const uint32_t d_tmem, const uint64_t adesc,
                                         const uint64_t bdesc, const uint32_t idesc,
                                         const uint32_t accumulate) {
    asm volatile("{\n\t.reg .pred p;\n\t"
                 "setp.ne.b32 p, %4, 0;\n\t"
                 "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n"
                 :: "r"(d_tmem), "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
                 : "memory");
}
// bar receives one arrival when every tcgen05 operation this thread issued
// before has completed
__device__ __forceinline__ void mma_commit(const uint32_t bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64"
                 " [%0];\n" :: "r"(bar) : "memory");
}

// 16 consecutive FP32 columns of the warp's 32 TMEM lanes (one lane per
// thread), then the wait for the load
__device__ __forceinline__ void tmem_ld16(const uint32_t taddr, float* v) {
    uint32_t r[16];
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x16.b32 "
                 "{%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15}, "
                 "[%16];\n"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]),
                   "=r"(r[6]), "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]),
                   "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
                 : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
#pragma unroll
    for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

// Shared-memory matrix descriptor of a K-major operand tile stored with the
// 128-byte swizzle: rows of 128 B (64 bf16 along K), 8-row groups 1024 B
// apart (stride byte offset), tile base 1024-byte aligned.  The k-th 16-wide
// K step of the tile starts 32 k bytes further (inside the swizzle atom).
__device__ __forceinline__ uint64_t desc_kmajor_sw128(const uint32_t saddr) {
    uint64_t d = 0;
    d |= (uint64_t)((saddr & 0x3FFFFu) >> 4);          // start address
    d |= (uint64_t)(16u >> 4) << 16;                    // leading byte offset
    d |= (uint64_t)(1024u >> 4) << 32;                  // stride byte offset
    d |= (uint64_t)1 << 46;                             // descriptor version
    d |= (uint64_t)2 << 61;                             // 128-byte swizzle
    return d;
}

// Instruction descriptor of kind::f16 with BF16 A and B (both K-major) and
// an FP32 accumulator, M x N
template<int M, int N>
__host__ __device__ constexpr uint32_t idesc_bf16_f32() {
    static_assert(M == 64 || M == 128, "M");
    static_assert(N % 16 == 0 && N >= 16 && N <= 256, "N");
    return (1u << 4)                      // D: FP32
         | (1u << 7)                      // A: BF16
         | (1u << 10)                     // B: BF16
         | ((uint32_t)(N >> 3) << 17)
         | ((uint32_t)(M >> 4) << 24);
}

}  // namespace tc
}  // namespace wb
