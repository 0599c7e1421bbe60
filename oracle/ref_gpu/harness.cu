// Launchers for the reference's own CUDA kernels (the GPU-side baseline).
//
// TEST INFRASTRUCTURE ONLY: compiled by oracle.build() into
// oracle/_ref/libref_gpu.so when the extracted kernel source
// oracle/_ref/ref_kernels.cuh exists (oracle/ref_gpu/extract.py); never
// linked into the product.  The kernels are the reference's, unmodified;
// this file only instantiates sgx_k_cls<LA, LB> (the reference's
// RawModule name expressions, gpu/sgx_k.py:468-482) and launches them with
// the reference's shapes: grid ceil(nsub / warps), block 32 * warps
// (gpu/sgx_k.py:764-780); the screen with 256-thread blocks over
// (sub-block, pair) (:890-902); the VV10 sum per 65,536-point chunk with
// 256-thread blocks (gpu/vv10.py:229-238).
#include <cuda_runtime.h>

#include "ref_kernels.cuh"

namespace {

typedef void (*ClsKernel)(const int*, const float*, const float*, const float*,
                          const float*, const int*, const double*, const float*,
                          const float*, const float*, const float*, const float*,
                          const float*, const float*, const float*, const float*,
                          const float*, const float*, const float*, const int*,
                          const int*, int, int, int, int, double, float*);

ClsKernel cls_kernel(int la, int lb) {
    switch (la * 4 + lb) {
    case 0: return sgx_k_cls<0, 0>;
    case 1: return sgx_k_cls<0, 1>;
    case 2: return sgx_k_cls<0, 2>;
    case 3: return sgx_k_cls<0, 3>;
    case 4: return sgx_k_cls<1, 0>;
    case 5: return sgx_k_cls<1, 1>;
    case 6: return sgx_k_cls<1, 2>;
    case 7: return sgx_k_cls<1, 3>;
    case 8: return sgx_k_cls<2, 0>;
    case 9: return sgx_k_cls<2, 1>;
    case 10: return sgx_k_cls<2, 2>;
    case 11: return sgx_k_cls<2, 3>;
    case 12: return sgx_k_cls<3, 0>;
    case 13: return sgx_k_cls<3, 1>;
    case 14: return sgx_k_cls<3, 2>;
    case 15: return sgx_k_cls<3, 3>;
    default: return sgx_k_tile;      // class 16: generally contracted pairs
    }
}

}  // namespace

extern "C" {

// the pair-table pointers of the reference's ShellPairsDevice, in its
// kernel argument order
struct RefPairs {
    const int* sh_dims;
    const float* sh_Mc;
    const float* sh_MT;
    const float* sh_Mc_lo;
    const float* sh_MT_lo;
    const int* pair_sh;
    const double* prim_p;
    const float* prim_prefac;
    const float* prim_prefac_lo;
    const float* prim_P_hi;
    const float* prim_P_lo;
    const float* prim_E;
};

// max threads per block of class cls (la * 4 + lb, 16 = generic), the
// attribute the reference sizes its blocks from
int ref_max_threads(int cls) {
    cudaFuncAttributes at;
    if (cudaFuncGetAttributes(&at, (const void*)cls_kernel(cls / 4, cls % 4)) != cudaSuccess)
        return -1;
    return at.maxThreadsPerBlock;
}

int ref_cls_launch(int cls, const RefPairs* P, const float* tp_hi, const float* tp_lo,
                   const float* cn_hi, const float* cn_lo, const float* coords,
                   const float* coords_lo, const float* F, const int* sub_off,
                   const int* sub_ids, int npts, int nao, int ks, int nsub,
                   double omega, float* G, int warps, void* stream) {
    if (nsub <= 0) return 0;
    ClsKernel k = cls == 16 ? (ClsKernel)sgx_k_tile : cls_kernel(cls / 4, cls % 4);
    k<<<(nsub + warps - 1) / warps, 32 * warps, 0, (cudaStream_t)stream>>>(
        P->sh_dims, P->sh_Mc, P->sh_MT, P->sh_Mc_lo, P->sh_MT_lo, P->pair_sh,
        P->prim_p, P->prim_prefac, P->prim_prefac_lo, P->prim_P_hi, P->prim_P_lo,
        P->prim_E, tp_hi, tp_lo, cn_hi, cn_lo, coords, coords_lo, F, sub_off,
        sub_ids, npts, nao, ks, nsub, omega, G);
    return (int)cudaGetLastError();
}

int ref_screen_launch(const float* cen, const float* rad, const float* msh,
                      const float* P, const float* pref, const float* pp,
                      const int* poff, const float* tau, const int* ish,
                      const int* jsh, int nsub, int npairs, int nbas,
                      float tol_over_safety, unsigned char* keep, void* stream) {
    const long long n = (long long)nsub * npairs;
    if (n <= 0) return 0;
    sgx_screen_mask<<<(unsigned)((n + 255) / 256), 256, 0, (cudaStream_t)stream>>>(
        cen, rad, msh, P, pref, pp, poff, tau, ish, jsh, nsub, npairs, nbas,
        tol_over_safety, keep);
    return (int)cudaGetLastError();
}

int ref_vv10_launch(const float* xyz, const float* q, const float* w0,
                    const float* kap, int n, double* F, double* U, double* W,
                    void* stream) {
    const int chunk = 65536, tile = 256;
    for (int i0 = 0; i0 < n; i0 += chunk) {
        const int i1 = i0 + chunk < n ? i0 + chunk : n;
        vv10_kernel_sum<<<(i1 - i0 + tile - 1) / tile, tile, 0, (cudaStream_t)stream>>>(
            xyz, q, w0, kap, n, i0, i1, F, U, W);
        const cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) return (int)e;
    }
    return 0;
}

}  // extern "C"
