// Fused screen + G kernel of one shell-pair class (included by the
// cosx_kernels_*.cu translation units, which pick the classes).
//
// One warp owns one 32-point sub-block at a time (one grid point per lane)
// and walks the class's shell pairs in ascending (A, B) order: 32 pairs at
// a time every lane evaluates one pair's screening bound (its header, shell
// maxima and tau were fetched one chunk ahead), a ballot compacts the kept
// ones, and the warp then runs each kept task with all lanes.  Headers come
// by shuffle; while one task computes, the next task's F_B (and its F_A
// when it opens a new run) and its first primitive-pair record are already
// in flight.  Tasks with the same bra shell A form a run: F_A is read and
// G_A stored once per run.
//
// Each class writes its own partial G buffer (rows of its two angular
// momenta), so classes can run concurrently; a fixed-order sum over the
// class buffers forms G.  A warp takes the next sub-block from a per-class
// counter (dynamic load balance); every element of a class buffer is
// written by one lane in a fixed order, so results do not depend on the
// launch shape, the scheduling or the overlap of classes.
//
// The bound is the reference's locked estimate (gpu/sgx_k.py:35-46,
// :417-456): tau * sum_prim pref F_0(p' d_min^2) * max(msh_A, msh_B) with
// d_min shrunk by 1e-5 (d + r) + 1e-6 and tol already divided by 1.001.
#pragma once
#include "launch.hpp"
#include "cosx_device.cuh"
#include "generated/cosx_layout.h"
#include "screen.cuh"

namespace wb {

constexpr int kCtaThreads = 128;
constexpr int kBoysFloat4 = 145 * 5;

// Minimum resident CTAs per SM requested per class (register cap
// 65536 / (128 * n)), one hex digit per class in class order (0,0), (1,0),
// (1,1), (2,0), ...; a build may override it with
// -DWB_COSX_MIN_BLOCKS=0x<10 hex digits>LL.
#ifndef WB_COSX_MIN_BLOCKS
#define WB_COSX_MIN_BLOCKS 0x6544331111LL
#endif
// the same for the dual-omega kernels (two sets of integrals and
// accumulators per lane): -DWB_COSX_MIN_BLOCKS2=0x<10 hex digits>LL
#ifndef WB_COSX_MIN_BLOCKS2
#define WB_COSX_MIN_BLOCKS2 0x5433321111LL
#endif
constexpr int min_blocks(int cls, int nw = 1) {
    long long v = nw == 2 ? WB_COSX_MIN_BLOCKS2 : WB_COSX_MIN_BLOCKS;
    for (int i = cls; i < kClasses - 1; ++i) v >>= 4;
    return (int)(v & 15) > 0 ? (int)(v & 15) : 1;
}

__device__ __forceinline__ int4 shfl_int4(const int4 v, int src) {
    return make_int4(__shfl_sync(0xffffffffu, v.x, src),
                     __shfl_sync(0xffffffffu, v.y, src),
                     __shfl_sync(0xffffffffu, v.z, src),
                     __shfl_sync(0xffffffffu, v.w, src));
}

// F rows n0 .. n0 + N - 1 at the point Fp points to (row stride ld)
template<int N>
__device__ __forceinline__ void load_f(const float* __restrict__ Fp,
                                       const int ld, const int n0, float* f) {
#pragma unroll
    for (int nu = 0; nu < N; ++nu) f[nu] = Fp[(long long)(n0 + nu) * ld];
}

// Record staging of one warp: two shared-memory buffers.  Lane form (the
// default): per-lane asynchronous 16-byte global -> shared copies
// (cp.async; the wait is the hardware's, no polling), lanes split the n
// float4.  TMA form (-DWB_COSX_TMA=1, two-omega kernels only): each buffer
// is filled with one TMA bulk copy (cp.async.bulk, global -> shared) that
// completes on the buffer's own mbarrier (expect_tx by lane 0, every lane
// waits on the phase parity).  Measured on the water27 bench step, the TMA
// form made the G phase 2-3 % slower (73.6 vs 71.5 ms): a task's records
// are a few hundred bytes, below the size where one bulk copy beats 32
// lanes' 16-byte copies, and the bounded wait loop adds instructions.
__device__ __forceinline__ void stage_records(float4* dst,
                                              const float4* __restrict__ src,
                                              const int n, const int lane) {
    for (int j = lane; j < n; j += 32) {
        const unsigned d = (unsigned)__cvta_generic_to_shared(dst + j);
        asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n"
                     :: "r"(d), "l"(src + j) : "memory");
    }
    asm volatile("cp.async.commit_group;\n" ::: "memory");
}
__device__ __forceinline__ void stage_wait() {
    asm volatile("cp.async.wait_all;\n" ::: "memory");
    __syncwarp();
}

#ifndef WB_COSX_TMA
#define WB_COSX_TMA 0
#endif
#if WB_COSX_TMA
// A wait gives up after kStageSpins polls: it sets *status, and the warp
// stops waiting (its results are then wrong and the host reports the
// failure), so a lost completion cannot hang the kernel.
constexpr int kStageSpins = 1 << 16;

// the two mbarriers of each warp of a CTA (8 B each)
__shared__ unsigned long long g_stage_mbar[kCtaThreads / 32][2];

// bits 0, 1: the phase parity buffer 0 / 1 completes next; bit 2: a wait
// gave up
struct RecStager {
    unsigned state;
};

__device__ __forceinline__ unsigned stage_bar(const int b) {
    return (unsigned)__cvta_generic_to_shared(&g_stage_mbar[threadIdx.x >> 5][b]);
}

// lane 0 of each warp initialises its two mbarriers (count 1); the CTA's
// __syncthreads after the Boys table load publishes them
__device__ __forceinline__ RecStager stager_init(const int lane) {
    RecStager st;
    st.state = 0u;
    if (lane == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n"
                     :: "r"(stage_bar(0)) : "memory");
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n"
                     :: "r"(stage_bar(1)) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
    }
    return st;
}

// n float4 from src (16-byte aligned) into dst = buffer b, one bulk copy
__device__ __forceinline__ void tma_stage_records(const int b, float4* dst,
                                                  const float4* __restrict__ src,
                                                  const int n, const int lane) {
    if (lane == 0) {
        const unsigned bar = stage_bar(b);
        const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
        const unsigned bytes = 16u * (unsigned)n;
        // the warp's earlier reads of this buffer (ordered by the caller's
        // __syncwarp) come before the async-proxy write
        asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
        asm volatile("{\n\t.reg .b64 st;\n\t"
                     "mbarrier.arrive.expect_tx.shared::cta.b64 st, [%0], %1;\n\t}\n"
                     :: "r"(bar), "r"(bytes) : "memory");
        asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes"
                     " [%0], [%1], %2, [%3];\n"
                     :: "r"(d), "l"(src), "r"(bytes), "r"(bar) : "memory");
    }
}

// wait until buffer b's copy has landed
__device__ __forceinline__ void tma_stage_wait(RecStager& st, const int b,
                                               unsigned long long* status) {
    if (!(st.state & 4u)) {
        const unsigned bar = stage_bar(b);
        const unsigned par = (st.state >> b) & 1u;
        unsigned done = 0;
        for (int i = 0; i < kStageSpins && !done; ++i)
            asm volatile("{\n\t.reg .pred p;\n\t"
                         "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
                         "selp.u32 %0, 1, 0, p;\n\t}\n"
                         : "=r"(done) : "r"(bar), "r"(par) : "memory");
        if (!done) {
            st.state |= 4u;
            if (status) atomicOr(status, 1ull);
        }
    }
    st.state ^= 1u << b;
    __syncwarp();
}
#define WB_STAGER_PARAM , RecStager& stg
#define WB_STAGER_ARG , stg
#else
#define WB_STAGER_PARAM
#define WB_STAGER_ARG
#endif
// with WB_COSX_SPLIT: the buffer set a block item writes (0, 1) and the
// index its cost is recorded at
#if WB_COSX_SPLIT
#define WB_SPLIT_PARAM , const int hset, const int citem
#else
#define WB_SPLIT_PARAM
#endif

__device__ __forceinline__ int lo16(const int x) { return x & 0xffff; }
__device__ __forceinline__ int hi16(const int x) {
    return (int)((unsigned)x >> 16);
}

// Points per lane of each class (1, 2 or 4), one hex digit per class in
// class order: more points share the per-task and per-primitive-pair
// overhead of the light classes (tasks of one to a few primitive pairs) at
// the cost of registers and of a screen over larger blocks.  A build may
// override it with -DWB_COSX_PTS=0x<10 hex digits>LL.
#ifndef WB_COSX_PTS
#define WB_COSX_PTS 0x2222111111LL
#endif
constexpr int class_pts(int cls) {
    long long v = WB_COSX_PTS;
    for (int i = cls; i < kClasses - 1; ++i) v >>= 4;
    const int p = (int)(v & 15);
    return p >= 4 ? 4 : (p >= 2 ? 2 : 1);
}
// the same for the dual-omega kernels: -DWB_COSX_PTS2=0x<10 hex digits>LL
#ifndef WB_COSX_PTS2
#define WB_COSX_PTS2 0x2222111111LL
#endif
constexpr int class_pts2(int cls) {
    long long v = WB_COSX_PTS2;
    for (int i = cls; i < kClasses - 1; ++i) v >>= 4;
    const int p = (int)(v & 15);
    return p >= 4 ? 4 : (p >= 2 ? 2 : 1);
}
template<int LA, int LB, int NW = 1> struct ClassPts {
    static constexpr int value = NW == 2 ? class_pts2(LA * (LA + 1) / 2 + LB)
                                         : class_pts(LA * (LA + 1) / 2 + LB);
};

// One block (32 * PTS points) of one class kernel: every pair of the class
// (screen, tasks, G) for the points of block blk.  A is the argument block
// of the block's molecule; wstage / rmax the warp's record buffers (two of
// rmax float4) and sbuf the one in use; kept / flops / ints accumulate the
// counters of the warp (with the TMA form, stg holds the buffers' copy
// state).
template<int LA, int LB, bool FAR, bool STAGE, int NW>
__device__ __forceinline__ void cosx_class_block(
    const CosxArgs& A, const int pair_begin, const int pair_end, const int blk,
    const float4* __restrict__ stab, float4* wstage, const int rmax, int& sbuf,
    unsigned long long& kept, unsigned long long& flops,
    unsigned long long& ints WB_STAGER_PARAM WB_SPLIT_PARAM) {
    constexpr int CLS = LA * (LA + 1) / 2 + LB;
    constexpr int NCA = (LA + 1) * (LA + 2) / 2;
    constexpr int NA = 2 * LA + 1;
    constexpr int NB = 2 * LB + 1;
    constexpr int PTS = ClassPts<LA, LB, NW>::value;
    const int lane = threadIdx.x & 31;
    constexpr int RS = NW == 2 ? kRecStride2[CLS] : kRecStride[CLS];
    const float4* __restrict__ recc = NW == 2 ? A.rec2[CLS] : A.rec[CLS];
#if WB_COSX_SPLIT
    float* const g1 = hset ? A.GclsH[CLS] : A.Gcls[CLS];
    float* const g2 = hset ? A.Gcls2H[CLS] : A.Gcls2[CLS];
    float* Gcw[2] = {g1, NW == 2 ? g2 : g1};
#else
    float* Gcw[2] = {A.Gcls[CLS], NW == 2 ? A.Gcls2[CLS] : A.Gcls[CLS]};
#endif
    const int ld = (int)A.ld;
    const float tol = A.tol;
    const float4* __restrict__ bnd = A.bnd + A.pp_begin[CLS];
    const float* __restrict__ bpref = A.bpref + A.pp_begin[CLS];
    constexpr int LVL = PTS == 4 ? 2 : PTS - 1;
    const float4* __restrict__ blk_cr = A.blk_cr[LVL];
    const float* __restrict__ blk_msh = A.blk_msh[LVL];
    unsigned long long bfl = 0;     // model flops kept in this block
    // the lane's points: blk * 32 PTS + 32 p + lane (clamped to the
    // arrays; ok marks the ones that exist)
    const float* __restrict__ Fp[PTS];
    float* Gp[NW * PTS];
    bool ok[PTS];
    float gxh[PTS], gyh[PTS], gzh[PTS], gxl[PTS], gyl[PTS], gzl[PTS];
#pragma unroll
    for (int p = 0; p < PTS; ++p) {
        const int g0 = blk * (32 * PTS) + 32 * p + lane;
        ok[p] = g0 < ld;
        const int g = ok[p] ? g0 : ld - 1;
        Fp[p] = A.F + g;
#pragma unroll
        for (int w = 0; w < NW; ++w) Gp[w * PTS + p] = Gcw[w] + g;
        gxh[p] = A.gxyz_hi[g];
        gyh[p] = A.gxyz_hi[ld + g];
        gzh[p] = A.gxyz_hi[2 * (long long)ld + g];
        gxl[p] = A.gxyz_lo[g];
        gyl[p] = A.gxyz_lo[ld + g];
        gzl[p] = A.gxyz_lo[2 * (long long)ld + g];
    }
    const float4 cr = blk_cr[blk];
    // zero this block's columns of the class buffer(s) (each element
    // has this lane as its one writer, so later stores and reductions
    // follow in program order; replaces a memset pass over the buffers)
    {
        const int nrow = A.crow[CLS];
        for (int r = 0; r < nrow; ++r) {
#pragma unroll
            for (int c = 0; c < NW * PTS; ++c)
                if (ok[c % PTS]) Gp[c][(long long)r * ld] = 0.0f;
        }
    }
    const float* __restrict__ ms = blk_msh + (long long)blk * A.nvshell;
    const int rem = A.npts - blk * 32 * PTS;
    const int nvalid = rem < 32 * PTS ? (rem > 0 ? rem : 0) : 32 * PTS;
    const int nsb = (nvalid + 31) / 32;     // 32-point sub-blocks covered
    // run state: the current bra shell (packed header word), its class
    // buffer row, f0 and Xa; pendA / fan: F_A prefetched for a next run
    int curA = -1, ga0 = 0, pendA = -1;
    float f0[PTS * NCA], Xa[NW * PTS * NCA], fan[PTS * NA];
#pragma unroll
    for (int c = 0; c < PTS * NCA; ++c) f0[c] = 0.0f;
#pragma unroll
    for (int c = 0; c < NW * PTS * NCA; ++c) Xa[c] = 0.0f;
#pragma unroll
    for (int c = 0; c < PTS * NA; ++c) fan[c] = 0.0f;
    // screen inputs of the first chunk
    int4 nhl = make_int4(0, 0, 0, 0);
    float2 ntp = make_float2(0.0f, 0.0f);
    float nfm = 0.0f;
    {
        const int k = pair_begin + lane;
        if (k < pair_end) {
            nhl = A.khdr[k];
            ntp = A.ptau[k];
            const int2 sh = A.pshell[k];
            nfm = fmaxf(ms[sh.x], ms[sh.y]);
        }
    }
    for (int c0 = pair_begin; c0 < pair_end; c0 += 32) {
        const int k = c0 + lane;
        const int4 hl = nhl;
        const float2 tp = ntp;
        const float fm = nfm;
        // the next chunk's header, tau and shell pair, then (after this
        // chunk's screen) its shell maxima
        const int kn = k + 32;
        int2 nsh = make_int2(0, 0);
        if (kn < pair_end) {
            nhl = A.khdr[kn];
            ntp = A.ptau[kn];
            nsh = A.pshell[kn];
        }
        bool keep = k < pair_end;
        if (keep && tol > 0.0f)
            keep = screen_pair(tol, bnd, bpref, cr, hl, tp, fm);
        if (kn < pair_end) nfm = fmaxf(ms[nsh.x], ms[nsh.y]);
        unsigned mask = __ballot_sync(0xffffffffu, keep);
        if (!mask) continue;
        int4 hdr = shfl_int4(hl, __ffs(mask) - 1);
        float fb[PTS * NB];
#pragma unroll
        for (int p = 0; p < PTS; ++p)
            load_f<NB>(Fp[p], ld, lo16(hdr.y), fb + p * NB);
        CosxRec<LA, LB> rec;
        if constexpr (STAGE) {
            __syncwarp();       // the previous chunk's reads of the buffer
#if WB_COSX_TMA
            if constexpr (NW == 2) {
                tma_stage_records(sbuf, wstage + sbuf * rmax,
                                  recc + (long long)hdr.z * RS, (hdr.w & 0xffff) * RS,
                                  lane);
                tma_stage_wait(stg, sbuf, A.status);
            } else
#endif
            {
                stage_records(wstage + sbuf * rmax, recc + (long long)hdr.z * RS,
                              (hdr.w & 0xffff) * RS, lane);
                stage_wait();
            }
        } else {
            cosx_rec_load<FAR>(A, hdr.z, rec);
        }
        while (true) {
            if (hdr.x != curA) {
                if (curA >= 0) {
#pragma unroll
                    for (int c = 0; c < NW * PTS; ++c)
                        cosx_end<LA>(Gp[c], ga0, ld, ok[c % PTS], Xa + c * NCA);
                }
                curA = hdr.x;
                ga0 = hi16(hdr.x);
                if (pendA != curA) {
#pragma unroll
                    for (int p = 0; p < PTS; ++p)
                        load_f<NA>(Fp[p], ld, lo16(hdr.x), fan + p * NA);
                    pendA = curA;
                }
#pragma unroll
                for (int p = 0; p < PTS; ++p)
                    cosx_begin<LA>(fan + p * NA, f0 + p * NCA);
#pragma unroll
                for (int c = 0; c < NW * PTS * NCA; ++c) Xa[c] = 0.0f;
            }
            mask &= mask - 1;
            // prefetch the next kept task of this chunk (fan is free:
            // f0 of the current run is formed)
            const bool more = mask != 0u;
            int4 hn = hdr;
            float fbn[PTS * NB];
            if (more) {
                hn = shfl_int4(hl, __ffs(mask) - 1);
#pragma unroll
                for (int p = 0; p < PTS; ++p)
                    load_f<NB>(Fp[p], ld, lo16(hn.y), fbn + p * NB);
                if (hn.x != hdr.x) {
#pragma unroll
                    for (int p = 0; p < PTS; ++p)
                        load_f<NA>(Fp[p], ld, lo16(hn.x), fan + p * NA);
                    pendA = hn.x;
                }
                // the next task's records into the other buffer (the
                // last reads of it ended before the previous wait)
                if constexpr (STAGE) {
#if WB_COSX_TMA
                    if constexpr (NW == 2)
                        tma_stage_records(sbuf ^ 1, wstage + (sbuf ^ 1) * rmax,
                                          recc + (long long)hn.z * RS,
                                          (hn.w & 0xffff) * RS, lane);
                    else
#endif
                        stage_records(wstage + (sbuf ^ 1) * rmax,
                                      recc + (long long)hn.z * RS,
                                      (hn.w & 0xffff) * RS, lane);
                }
            }
            const int gb0 = hi16(hdr.y), pp0 = hdr.z, npp = hdr.w & 0xffff;
            const int nxt = more ? hn.z : pp0;
            if constexpr (NW == 2) {
                const float4* rp = wstage + sbuf * rmax;
                if constexpr (LA == LB) {
                    if (hdr.w >> 16)
                        CosxTask2<LA, LB, true, PTS>::run(
                            Gp, ld, gb0, rp, npp, ok, gxh, gyh, gzh,
                            gxl, gyl, gzl, stab, f0, fb, Xa);
                    else
                        CosxTask2<LA, LB, false, PTS>::run(
                            Gp, ld, gb0, rp, npp, ok, gxh, gyh, gzh,
                            gxl, gyl, gzl, stab, f0, fb, Xa);
                } else {
                    CosxTask2<LA, LB, false, PTS>::run(
                        Gp, ld, gb0, rp, npp, ok, gxh, gyh, gzh,
                        gxl, gyl, gzl, stab, f0, fb, Xa);
                }
            } else if constexpr (STAGE) {
                const float4* rp = wstage + sbuf * rmax;
                if constexpr (LA == LB) {
                    if (hdr.w >> 16)
                        CosxTask<LA, LB, true, PTS, FAR, true>::run(
                            A, Gp, ld, gb0, rp, npp, ok, gxh, gyh, gzh,
                            gxl, gyl, gzl, stab, f0, fb, Xa);
                    else
                        CosxTask<LA, LB, false, PTS, FAR, true>::run(
                            A, Gp, ld, gb0, rp, npp, ok, gxh, gyh, gzh,
                            gxl, gyl, gzl, stab, f0, fb, Xa);
                } else {
                    CosxTask<LA, LB, false, PTS, FAR, true>::run(
                        A, Gp, ld, gb0, rp, npp, ok, gxh, gyh, gzh,
                        gxl, gyl, gzl, stab, f0, fb, Xa);
                }
            } else if constexpr (LA == LB) {
                if (hdr.w >> 16)
                    CosxTask<LA, LB, true, PTS, FAR, false>::run(
                        A, Gp, ld, gb0, pp0, npp, nxt, ok, gxh, gyh, gzh,
                        gxl, gyl, gzl, stab, f0, fb, Xa, rec);
                else
                    CosxTask<LA, LB, false, PTS, FAR, false>::run(
                        A, Gp, ld, gb0, pp0, npp, nxt, ok, gxh, gyh, gzh,
                        gxl, gyl, gzl, stab, f0, fb, Xa, rec);
            } else {
                CosxTask<LA, LB, false, PTS, FAR, false>::run(
                    A, Gp, ld, gb0, pp0, npp, nxt, ok, gxh, gyh, gzh,
                    gxl, gyl, gzl, stab, f0, fb, Xa, rec);
            }
            kept += nsb * NW;
            if (!more) break;
            if constexpr (STAGE) {
#if WB_COSX_TMA
                if constexpr (NW == 2)
                    tma_stage_wait(stg, sbuf ^ 1, A.status);
                else
#endif
                    stage_wait();
                sbuf ^= 1;
            }
            hdr = hn;
#pragma unroll
            for (int nu = 0; nu < PTS * NB; ++nu) fb[nu] = fbn[nu];
        }
        // model flops / integrals of the kept tasks of this chunk
        if (keep) {
            const unsigned long long fk =
                (unsigned long long)A.pflops[k] * nvalid * NW;
            flops += fk;
            bfl += fk;
            ints += (unsigned long long)A.pnint[k] * nvalid * NW;
        }
    }
    if (curA >= 0) {
#pragma unroll
        for (int c = 0; c < NW * PTS; ++c)
            cosx_end<LA>(Gp[c], ga0, ld, ok[c % PTS], Xa + c * NCA);
    }
    for (int o = 16; o > 0; o >>= 1) bfl += __shfl_xor_sync(0xffffffffu, bfl, o);
#if WB_COSX_SPLIT
    if (lane == 0 && A.bcost[CLS]) A.bcost[CLS][citem] = (float)bfl;
#else
    if (lane == 0 && A.bcost[CLS]) A.bcost[CLS][blk] = (float)bfl;
#endif
}

template<int LA, int LB, bool FAR, bool STAGE, int NW>
__global__ void __launch_bounds__(kCtaThreads,
                                  min_blocks(LA * (LA + 1) / 2 + LB, NW))
cosx_class_kernel(const CosxArgs A, const int pair_begin, const int pair_end) {
    static_assert(NW == 1 || (NW == 2 && STAGE), "dual-omega needs staging");
    constexpr int CLS = LA * (LA + 1) / 2 + LB;
    constexpr int PTS = ClassPts<LA, LB, NW>::value;
    __shared__ float4 stab[kBoysFloat4];
#if WB_COSX_TMA
    RecStager stg = stager_init(threadIdx.x & 31);
#endif
    for (int i = threadIdx.x; i < kBoysFloat4; i += blockDim.x)
        stab[i] = A.boys[i];
    __syncthreads();
    const int lane = threadIdx.x & 31;
    // STAGE: per warp, two record buffers of recmax float4 (dynamic smem)
    extern __shared__ float4 s_stage[];
    const int rmax = NW == 2 ? A.recmax2[CLS] : A.recmax[CLS];
    float4* wstage = s_stage + (threadIdx.x >> 5) * 2 * rmax;
    int sbuf = 0;
    constexpr int LVL = PTS == 4 ? 2 : PTS - 1;
    const int nblk = A.nblk[LVL];
    unsigned long long kept = 0, flops = 0, ints = 0;
    const int* __restrict__ order = A.border[CLS];
#if WB_COSX_SPLIT
    // items 2 blk + h: half h of block blk
    const int nitem = 2 * nblk;
    const int split = A.cls_split[CLS];
    for (;;) {
        int item = 0;
        if (lane == 0) item = atomicAdd(A.work + CLS, 1);
        item = __shfl_sync(0xffffffffu, item, 0);
        if (item >= nitem) break;
        int it = item;
        if (order) {
            const int b = order[item];
            it = b >= 0 && b < nitem ? b : item;
        }
        const int blk = it >> 1, h = it & 1;
        cosx_class_block<LA, LB, FAR, STAGE, NW>(A, h ? split : pair_begin,
                                                 h ? pair_end : split, blk, stab,
                                                 wstage, rmax, sbuf, kept, flops,
                                                 ints WB_STAGER_ARG, h, it);
    }
#else
    for (;;) {
        int item = 0;
        if (lane == 0) item = atomicAdd(A.work + CLS, 1);
        item = __shfl_sync(0xffffffffu, item, 0);
        if (item >= nblk) break;
        // costliest blocks first (the order is a permutation of 0 .. nblk-1)
        int blk = item;
        if (order) {
            const int b = order[item];
            blk = b >= 0 && b < nblk ? b : item;
        }
        cosx_class_block<LA, LB, FAR, STAGE, NW>(A, pair_begin, pair_end, blk, stab,
                                                 wstage, rmax, sbuf, kept, flops,
                                                 ints WB_STAGER_ARG);
    }
#endif
    // lane 0 counted the tasks (every lane runs every task) in units of the
    // 32-point sub-blocks they cover; every lane counted the flops /
    // integrals of its own pairs
    for (int o = 16; o > 0; o >>= 1) {
        flops += __shfl_xor_sync(0xffffffffu, flops, o);
        ints += __shfl_xor_sync(0xffffffffu, ints, o);
    }
    if (lane == 0 && kept) {
        atomicAdd(A.counters + 3 * CLS + 0, kept);
        atomicAdd(A.counters + 3 * CLS + 1, flops);
        atomicAdd(A.counters + 3 * CLS + 2, ints);
    }
}

// Batched form: the blocks of one class over several molecules in one
// launch.  args[m] is molecule m's argument block (its class pair range in
// cls_pb / cls_pe); its blocks of this class are the items item_off[m] ..
// item_off[m + 1] - 1 (ascending).  Warps take items from one counter
// (*work) and copy the argument block of the molecule they work on into
// shared memory; rmax is the largest task record of the class over the
// molecules (the dynamic shared memory holds two per warp).  order, if not
// null, is the order in which the items are taken (costliest first, from
// the block costs the previous launch recorded through each molecule's
// bcost).  The Boys table
// is the same for every molecule.  Each molecule's counters receive its own
// tasks; every element of every class buffer keeps one writer lane and its
// summation order, so each molecule's G equals its single-molecule G.
template<int LA, int LB, bool FAR, bool STAGE, int NW>
__global__ void __launch_bounds__(kCtaThreads,
                                  min_blocks(LA * (LA + 1) / 2 + LB, NW))
cosx_class_kernel_batch(const CosxArgs* __restrict__ args,
                        const int* __restrict__ item_off, const int nmol,
                        int* __restrict__ work, const int rmax,
                        const int* __restrict__ order) {
    static_assert(NW == 1 || (NW == 2 && STAGE), "dual-omega needs staging");
    constexpr int CLS = LA * (LA + 1) / 2 + LB;
    constexpr int NWARP = kCtaThreads / 32;
    static_assert(sizeof(CosxArgs) % 4 == 0, "argument block copied as words");
    __shared__ float4 stab[kBoysFloat4];
    __shared__ CosxArgs sA[NWARP];
    const int lane = threadIdx.x & 31;
    const int warp = threadIdx.x >> 5;
#if WB_COSX_TMA
    RecStager stg = stager_init(lane);
#endif
    const float4* __restrict__ boys = args[0].boys;
    for (int i = threadIdx.x; i < kBoysFloat4; i += blockDim.x) stab[i] = boys[i];
    __syncthreads();
    extern __shared__ float4 s_stage[];
    float4* wstage = s_stage + warp * 2 * rmax;
    int sbuf = 0;
    const int total = item_off[nmol];
    int cur = -1;
    unsigned long long kept = 0, flops = 0, ints = 0;
    auto flush = [&]() {
        unsigned long long f = flops, n = ints;
        for (int o = 16; o > 0; o >>= 1) {
            f += __shfl_xor_sync(0xffffffffu, f, o);
            n += __shfl_xor_sync(0xffffffffu, n, o);
        }
        if (lane == 0 && kept) {
            unsigned long long* c = sA[warp].counters + 3 * CLS;
            atomicAdd(c + 0, kept);
            atomicAdd(c + 1, f);
            atomicAdd(c + 2, n);
        }
        kept = flops = ints = 0;
    };
    for (;;) {
        int item = 0, m = 0;
        if (lane == 0) {
            item = atomicAdd(work, 1);
            if (item < total) {
                // costliest items first (a permutation of 0 .. total - 1)
                if (order) {
                    const int o = order[item];
                    item = o >= 0 && o < total ? o : item;
                }
                int lo = 0, hi = nmol;          // item_off[lo] <= item < item_off[hi]
                while (hi - lo > 1) {
                    const int mid = (lo + hi) >> 1;
                    if (item_off[mid] <= item) lo = mid; else hi = mid;
                }
                m = lo;
            }
        }
        item = __shfl_sync(0xffffffffu, item, 0);
        if (item >= total) break;
        m = __shfl_sync(0xffffffffu, m, 0);
        if (m != cur) {
            if (cur >= 0) flush();
            __syncwarp();
            const int* src = reinterpret_cast<const int*>(args + m);
            int* dst = reinterpret_cast<int*>(sA + warp);
            for (int i = lane; i < (int)(sizeof(CosxArgs) / 4); i += 32) dst[i] = src[i];
            __syncwarp();
            cur = m;
        }
        const CosxArgs& Am = sA[warp];
#if WB_COSX_SPLIT
        // two items per block, as in the single-molecule kernel: half h of
        // block it >> 1 writes buffer set h (summed after set 0)
        {
            const int it = item - item_off[m];
            const int h = it & 1;
            const int split = Am.cls_split[CLS];
            cosx_class_block<LA, LB, FAR, STAGE, NW>(Am, h ? split : Am.cls_pb[CLS],
                                                     h ? Am.cls_pe[CLS] : split,
                                                     it >> 1, stab, wstage, rmax, sbuf,
                                                     kept, flops, ints WB_STAGER_ARG,
                                                     h, it);
        }
#else
        cosx_class_block<LA, LB, FAR, STAGE, NW>(Am, Am.cls_pb[CLS], Am.cls_pe[CLS],
                                                 item - item_off[m], stab, wstage,
                                                 rmax, sbuf, kept, flops,
                                                 ints WB_STAGER_ARG);
#endif
    }
    if (cur >= 0) flush();
}

}  // namespace wb
