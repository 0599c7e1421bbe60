// Argument blocks and launchers of the SCF kernels (scf_kernels.cu).
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace wb {
namespace scf {

// one-electron integrals over the physical shells (AO-evaluation tables)
struct Int1eArgs {
    int nbas, nao;
    const int* sh_l;
    const int* sh_np;
    const int* sh_nc;
    const int* sh_eoff;
    const int* sh_coff;
    const int* sh_ao0;
    const double* sh_ctr;       // (nbas, 3), handle frame
    const double* exps;
    const double* coeffs;
    int natm;
    const double* nuc_xyz;      // (natm, 3), handle frame
    const double* nuc_z;        // (natm,) nuclear charges
    const double* boys;         // FP64 Boys table (kBoys64Nodes x kBoys64Cols)
    double* S;                  // (nao, nao) row-major outputs
    double* T;
    double* V;
};

// Hermite densities of the primitive pairs for one density matrix
struct DhArgs {
    int npairs, nao;
    const double* D;            // (nao, nao) row-major, symmetric
    const int4* hdr;            // per pair: ia0, ib0, pp0, npp | diag << 16
    const int* pclass;          // per pair: class (la, lb)
    const int* pcls_l;          // per pair: class index (kernel dispatch)
    const double* E;            // FP64 E blocks of the classes
    long long e_base[10];
    int pp_begin[10];
    const double* pref;         // per primitive pair: folded prefactor
    const long long* dh_off;    // per primitive pair: offset of its density
    double* dh64;
    float* dh32;
    float* pair_dabs;           // per pair: w sum |D_AB| (rounded up)
};

struct HartreeArgs {
    const double* coords;       // (npts, 3) handle frame
    int64_t npts;
    const float4* blk_cr;       // per 32-point block
    int nblk;
    int npairs;
    const int4* hdr;
    const int* pair_L;
    const float2* ptau;
    const float4* bnd;          // per primitive pair (global index)
    const float* bpref;
    const float* pair_dabs;
    const double* P;            // per primitive pair, FP64
    const double* p;
    const float4* geo;          // per primitive pair: P hi, P lo (FP32)
    const float* p32;
    const long long* dh_off;
    const double* dh64;
    const float* dh32;
    const float4* boys32;
    const double* boys64;
    float tol;                  // screening tolerance / 1.001 (0 keeps all)
    double* v;                  // (npts,) output
    int* work;                  // zeroed block counter
    unsigned long long* kept;   // kept (block, pair) tasks, or null
};

cudaError_t upload_int1e_c2s(const double* all110);
cudaError_t launch_int1e(const Int1eArgs& a, cudaStream_t s);
cudaError_t launch_dh(const DhArgs& a, cudaStream_t s);
cudaError_t launch_block_geom(const double* xyz, int64_t npts, int nblk, float4* cr,
                              cudaStream_t s);
cudaError_t launch_hartree(const HartreeArgs& a, bool fp64, cudaStream_t s);

}  // namespace scf
}  // namespace wb
