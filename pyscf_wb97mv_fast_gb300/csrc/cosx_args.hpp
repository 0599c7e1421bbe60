// Argument block of the fused COSX class kernels (host + device visible).
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

// WB_COSX_SPLIT = 1 (the default): each point block of a class is two work
// items, its pair range cut at a run boundary near the middle of the
// class's model flops; the second half writes a second set of class
// buffers, summed after the first.  Twice the items per warp for the load
// balance of the heavy classes, bitwise reproducible.  Measured on the
// water27 bench step (384,435 points): G phase 68.5 ms against 71.7 ms
// with -DWB_COSX_SPLIT=0 (one item per block).
#ifndef WB_COSX_SPLIT
#define WB_COSX_SPLIT 1
#endif

namespace wb {

constexpr int kClasses = 10;

// Everything one class launch reads.  Per primitive pair m (global index):
//   geo[2m], geo[2m+1]   P hi (xyz, 0), P lo (xyz, 0)      molecule frame
//   om[5m .. 5m+4]       tp_hi, tp_lo, c0_hi, c0_lo, ..., c6_hi, c6_lo,
//                        K0_hi, K0_lo, r^2 far-field threshold, 0
//   Ecls[c] + (m - pp_begin[c]) * stride_c/4   packed Hermite E
// Per pair k: hdr[k] = (ia0, ib0, pp0, npp | diag << 16), khdr[k] = (ia0 |
// ga0 << 16, ib0 | gb0 << 16, pp0, npp | diag << 16) with ga0 / gb0 the
// rows of A / B in the class's partial-G buffer, pshell[k] = (virtual shell
// A, B), ptau[k] = (tau, tau * sum pref).
struct CosxArgs {
    const float* F;            // (nao, ld) AO-major, FP32
    float* Gcls[kClasses];     // per class (rows, ld) partial G; each class
                               // kernel zeroes its block's columns first
    int crow[kClasses];        // rows of each class buffer
    long long ld;              // padded point count (multiple of 32)
    int npts;                  // valid points
    int nsub;                  // ld / 32
    const float4* geo;
    const float4* om;
    // per class, packed per primitive pair (class-local index m):
    // rec[c] + m * stride_c = P hi, P lo, omega record (n_om float4), E
    const float4* rec[kClasses];
    int recmax[kClasses];      // float4 of the largest task record per class
    // dual-omega launches: records of two omegas per pair (stride 2 + 2 n_om
    // + n_e), and the second omega's class buffers
    const float4* rec2[kClasses];
    int recmax2[kClasses];
    float* Gcls2[kClasses];
    const float4* Ecls[kClasses];
    int pp_begin[kClasses];
    const int4* hdr;
    const int4* khdr;
    const int2* pshell;
    const float2* ptau;
    const float4* bnd;         // per pp: P (FP32), p' = 0.75 p
    const float* bpref;        // per pp: bound prefactor (rounded up)
    // per block of 32 * PTS points (index log2 PTS): centroid (xyz), radius
    // and msh (nblk, nvshell) = max_g w_g sum_shell |F|
    const float4* blk_cr[3];
    const float* blk_msh[3];
    int nblk[3];
    int nvshell;
    float tol;                 // tile_tol / 1.001, <= 0 keeps every task
    const float* gxyz_hi;      // (3, ld) SoA grid coordinates, hi
    const float* gxyz_lo;      // (3, ld) lo
    const float4* boys;        // Boys table, BOYS_NODES rows of 5 float4
    const long long* pflops;   // per pair model flops per point
    const int* pnint;          // per pair nfi * nfj
    unsigned long long* counters;  // per class: kept, flops, ints (3 each)
    int* work;                 // per class dynamic sub-block counter
    // block order: the i-th block a class kernel takes is border[c][i]
    // (a permutation of its blocks, costliest first; nullptr = ascending),
    // and bcost[c][blk] receives the model flops of the tasks block blk
    // kept (the order of the next call on the same grid)
    const int* border[kClasses];
    float* bcost[kClasses];
    // the class pair ranges (the batched kernels read them from here)
    int cls_pb[kClasses];
    int cls_pe[kClasses];
    unsigned long long* status;    // nonzero: a record staging wait gave up
#if WB_COSX_SPLIT
    float* GclsH[kClasses];    // class buffers of the second half of each block
    float* Gcls2H[kClasses];
    int cls_split[kClasses];   // first pair of the second half
#endif
};

}  // namespace wb
