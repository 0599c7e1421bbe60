// Device-side pieces of the fused COSX exchange kernel family (sm_103a):
// the per-class task bodies (generated/cosx_classes.cuh).
#pragma once
#include "cosx_args.hpp"
#include "boys.cuh"

namespace wb {

// The inputs of one primitive pair a class reads (geo, omega record and,
// for small classes, the Hermite E record), held in registers one pair
// ahead of the computation.
template<int LA, int LB> struct CosxRec;
// (one overload per class, generated: cosx_rec_load<FAR>(A, m, rec))

// One task of class (LA, LB) on PTS grid points per lane (arrays of PTS:
// Gp = the point's column of the class buffer (row stride ld; points past
// the array are clamped to its last column), ok = the point exists, its
// coordinates): loop over the class-local primitive pairs pp0 .. pp0 +
// npp - 1, G_B update in rows gb0 .. of the class buffer, bra-side
// Cartesian accumulators Xa
// (PTS x NCA) carried across the run of tasks with the same A.  rec holds
// pair pp0's record on entry and pair nxt's on exit (the next task's first
// pair).  The DIAG form (B = A) adds its ket accumulators to Xa instead of
// writing G_B.  FAR selects the order of the warp-uniform R000 branches:
// all-far first (T >= 36 common: omega = 0) or all-near first (long-range
// omegas, where theta p <= omega^2 keeps T small); mixed warps choose per
// point between the far-field form and the Boys Taylor form.  STAGE: the task's primitive-pair records were
// copied to shared memory (rp, stride per class) instead of being carried
// in registers one pair ahead.  Specialised per (LA, LB, DIAG, FAR,
// STAGE) with run() as the body.
template<int LA, int LB, bool DIAG, int PTS, bool FAR, bool STAGE> struct CosxTask;

// The same task for two omegas at once (records staged in shared memory,
// dual layout): distances, headers and F shared; integrals, accumulators
// and G_B per omega slot w (Gp[w * PTS + p], Xa[(w * PTS + p) * NCA ..]).
template<int LA, int LB, bool DIAG, int PTS> struct CosxTask2;

// Start of a run: f0 = c2s^T F_A (Cartesian components of F on shell A).
template<int LA>
__device__ __forceinline__ void cosx_begin(const float* fa, float* f0);

// End of a run: G_A = c2s^T Xa, stored to rows ga0 .. of the class buffer
// at the point Gp points to (row stride ld), if the point exists.
template<int LA>
__device__ __forceinline__ void cosx_end(float* __restrict__ Gp, const int ga0,
                                         const int ld, const bool ok,
                                         const float* Xa);

// G_B += y for the ket rows of a task: a reduction in L2 (red.global.add,
// no value returned), so the task neither waits for nor holds the old
// value.  Every element of a class buffer has one writer lane, whose
// operations on one address take effect in program order: the sum order,
// and so the result, is the same as a load-add-store (the reduction
// flushes subnormal results to zero).  -DWB_COSX_GB_RED=0 selects the
// load-add-store.
#ifndef WB_COSX_GB_RED
#define WB_COSX_GB_RED 1
#endif
__device__ __forceinline__ void gb_add(float* p, const float y) {
    atomicAdd(p, y);
}

// Packed FP32 (f32x2.cuh) in the PTS = 2 two-omega task bodies: the
// distances, far-field R000, recurrences, Hermite sums and accumulations
// of the lane's two points in float2 halves (the near-field Boys sums stay
// per point: each point reads its own table row).  -DWB_COSX_F32X2=0
// compiles the scalar form.
#ifndef WB_COSX_F32X2
#define WB_COSX_F32X2 1
#endif

}  // namespace wb

namespace wb {
#include "generated/cosx_classes.cuh"
}
