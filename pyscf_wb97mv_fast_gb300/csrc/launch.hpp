// Kernel launchers shared between the CUDA translation units and the C ABI.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#include "cosx_args.hpp"

namespace wb {

// SMs of the current device (cached per device; 152 on a GB300).
inline int sm_count() {
    static int cached[64] = {};
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return 152;
    if (!cached[dev]) {
        int n = 0;
        if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
            n <= 0)
            return 152;
        cached[dev] = n;
    }
    return cached[dev];
}

// Blocks of a grid-stride loop over n items: enough for every item, capped
// at ctas_per_sm resident blocks per SM of the current device.
inline int64_t grid_stride_blocks(int64_t n, int threads, int ctas_per_sm) {
    const int64_t want = (n + threads - 1) / threads;
    const int64_t cap = (int64_t)sm_count() * ctas_per_sm;
    return want < 1 ? 1 : (want < cap ? want : cap);
}

// per-class fused screen + G kernels (cosx_kernels_*.cu); far selects the
// variant with the far-field R000 form (omega = 0, where T >= 36 is common);
// stage_smem > 0 selects the variant that stages each task's primitive-pair
// records in shared memory (stage_smem bytes of dynamic smem per CTA)
// dual runs the dual-omega variant (two omegas per launch, staged records
// of the dual layout; far is then unused)
cudaError_t launch_cosx_class_range(int cls, const CosxArgs& a, int pb,
                                    int pe, int grid, cudaStream_t s, bool far,
                                    size_t stage_smem, bool dual = false);
// the batched form: one launch over the class's blocks of nmol molecules
// (args: nmol device argument blocks; off: nmol + 1 item offsets; work: a
// zeroed counter; rmax: the largest task record of the class over the
// molecules, smem = 4 warps x 2 x rmax float4 when staged; order: the item
// order, costliest first, or null for ascending)
cudaError_t launch_cosx_class_batch(int cls, const CosxArgs* args, const int* off,
                                    int nmol, int* work, int rmax, const int* order,
                                    int grid, cudaStream_t s, bool far, size_t smem,
                                    bool dual);
// max resident CTAs per SM of a class kernel (128 threads each); 0 if the
// kernel cannot run with that much dynamic shared memory
int cosx_class_blocks_per_sm(int cls, bool far, size_t stage_smem,
                             bool dual = false);

struct AoArgs {
    const double* coords;       // (npts, 3) molecule frame
    int64_t npts, ld;
    int nbas;
    const int* sh_l;
    const int* sh_np;
    const int* sh_nc;
    const int* sh_eoff;
    const int* sh_coff;
    const int* sh_ao0;
    const double* sh_ctr;       // (nbas, 3)
    const double* exps;
    const double* coeffs;
    double* X;                  // (nao, ld), or (4, nao, ld) for deriv 1
    int nao;
};

cudaError_t launch_ao_eval(const AoArgs& a, cudaStream_t s);
cudaError_t launch_ao_eval_d1(const AoArgs& a, cudaStream_t s);
cudaError_t upload_c2s_tables(const double* t0, const double* t1,
                              const double* t2, const double* t3);
cudaError_t upload_c2s_f(const float* all /* 4 x 70 */);
// 2^(-j/64), j = 0..63, for the AO kernels' exp
cudaError_t upload_exp_table(const double* t64);

// class ranges and record layout for launch_pack_records (classes with no
// primitive pairs have pp_begin == pp_end)
struct RecPack {
    int pp_begin[10], pp_end[10], stride[10], nom[10], ne[10];
    long long rec_off[10];      // float4 offset of the class's records
    long long e_off[10];        // float4 offset of the class's E block
};
cudaError_t launch_pack_records(const RecPack& P, int npp, const float4* geo,
                                const float4* om, const float4* E,
                                float4* rec, cudaStream_t s);
// dual-omega records: geo, the first n_om - 1 float4 and the far-field
// float4 of om_a, then the same of om_b, then E (P.stride = dual stride)
cudaError_t launch_pack_records2(const RecPack& P, int npp, const float4* geo,
                                 const float4* om_a, const float4* om_b,
                                 const float4* E, float4* rec, cudaStream_t s);
cudaError_t launch_omega(int npp, const double* p, const double* pref,
                         double omega, float4* om, cudaStream_t s);
cudaError_t launch_grid_prep(const double* coords, int64_t npts, int64_t ld,
                             float* hi, float* lo, cudaStream_t s);
// centroid / radius and shell maxima per block of 32, 64 and 128 points
// (level k = 0, 1, 2: ceil(ld / (32 2^k)) blocks), one pass over F
struct BlockStatsOut {
    float4* cr[3];
    float* msh[3];
};
cudaError_t launch_sub_stats(const double* coords, const double* weights,
                             const float* F, int64_t npts, int64_t ld,
                             int nvshell, const int* vs_ao0, const int* vs_nf,
                             const BlockStatsOut& out, cudaStream_t s);
// points per lane (1, 2 or 4) of a class kernel: its blocks hold 32 * pts
int cosx_class_pts(int cls, bool dual = false);
cudaError_t launch_f64_to_f32(const double* in, float* out, int64_t n,
                              cudaStream_t s);
// G = fixed-order sum of the class partial-G rows (4 source rows per AO)
// block order of each class from the per-block costs of a previous launch
// (cost / order: kClasses rows of stride floats / ints; n[c] blocks of class
// c, 0 = leave the class alone)
struct BlockOrderArgs {
    const float* cost;
    int* order;
    long long stride;
    int n[kClasses];
};
cudaError_t launch_block_order(const BlockOrderArgs& P, cudaStream_t s);
// semilocal XC: density parameters (5, ld) FP64 and the Fock-side planes
cudaError_t launch_xc_rho(const double* X, const float* T, int nao, int64_t ld,
                          int64_t npts, int mgga, double* rho, cudaStream_t s);
cudaError_t launch_xc_aow(const double* X, const double* v, int nao, int64_t ld,
                          int64_t npts, int mgga, float* G, cudaStream_t s);
cudaError_t launch_gsum(const float* gc, const int4* src, int nao, int64_t ld,
                        float* G, cudaStream_t s);
// the same over two buffer sets (the halves of split blocks), gc0 first
cudaError_t launch_gsum2(const float* gc0, const float* gc1, const int4* src, int nao,
                         int64_t ld, float* G, cudaStream_t s);
cudaError_t launch_weight_g(const float* G, const double* w, int64_t npts,
                            int64_t ld, int nao, double* out, cudaStream_t s);
cudaError_t launch_dense_impl(const CosxArgs& a, int npairs, const int* pclass,
                              const int* pl, const int* estride, int nao,
                              float* out, cudaStream_t s);
// the fused screen alone: keep (a.nblk[lv], npairs) uint8 (test aid)
cudaError_t launch_screen_mask(const CosxArgs& a, int lv, int npairs,
                               unsigned char* keep, cudaStream_t s);
cudaError_t launch_boys(const float* t, int64_t n, int nmax,
                        const float4* tab, float* out, cudaStream_t s);
// VV10 double sum; ws must hold vv10_workspace_bytes(n) bytes
size_t vv10_workspace_bytes(int64_t n);
// packed: fma.rn.f32x2 (two FP32 FMAs per instruction) instead of fmaf
cudaError_t launch_fma_probe(int64_t iters, int blocks, int threads,
                             float* out, cudaStream_t s, bool packed = false);
// batched VV10: tiles of several molecules (see vv10.cu); device arrays
struct VvSeg {
    const long long* tstart;    // first point of each tile
    const int* tlen;            // points of each tile (1 .. 256)
    const int* tmol;            // molecule of each tile
    const int* mtile;           // nmol + 1: first tile of each molecule
    long long ntiles;
};
size_t vv10_tile_stats_bytes(int64_t ntiles);
// stats: vv10_tile_stats_bytes(ntiles) bytes; kept: a zeroed counter or null
cudaError_t launch_vv10_seg(const float* xyz, const float* q, const float* w0,
                            const float* kap, const VvSeg& sg, double tile_tol,
                            double* F, double* U, double* W, void* stats,
                            unsigned long long* kept, cudaStream_t s);
cudaError_t launch_vv10(const float* xyz, const float* q, const float* w0,
                        const float* kap, int64_t n, double tile_tol,
                        double* F, double* U, double* W, void* ws,
                        cudaStream_t s);

}  // namespace wb
