// Integral-derivative part of the COSX exchange gradient (cosx_grad64.cu):
// argument block and launchers.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace wb {

struct CosxGradArgs {
    const double* F;            // (nao, ld) AO-major, FP64: F = X D
    const double* coords;       // (npts, 3) molecule frame
    const double* weights;      // (npts,)
    long long ld;
    int npts;
    double omega;
    // the screen of the FP64 kernels (32-point blocks)
    const int4* khdr;
    const int2* pshell;
    const float2* ptau;
    const float4* bnd;
    const float* bpref;
    const float4* blk_cr;
    const float* blk_msh;
    int nblk;
    int nvshell;
    float tol;
    int pp_begin[10];
    // FP64 pair data: per primitive pair P (3), p, folded prefactor, bra
    // exponent; per virtual shell its centre (3) and atom
    const double* P;
    const double* p;
    const double* pref;
    const double* alpha;
    const double* vs_xyz;
    const int* vs_atom;
    const double* boys;         // kBoys64Nodes x kBoys64Cols
    const double* c2s;          // l = 2 at 0, l = 3 at 30
    double* gbuf;               // (nblk, natm, 3) per-block partial gradients
    int natm;
    int* work;                  // per class block counter (zeroed)
};

cudaError_t launch_cosx_grad64_class(int cls, const CosxGradArgs& a, int pb, int pe,
                                     int nsm, cudaStream_t s);
// out (natm * 3) += sum over the nblk rows of gbuf, in row order
cudaError_t launch_grad_rows_sum(const double* gbuf, int nblk, int natm, double* out,
                                 cudaStream_t s);
// out (nao, 3): sum_g w_g dX[x][mu][g] H[mu][g] (fixed-order block reduction)
cudaError_t launch_ao_dot(const double* dX, const double* H, const double* w,
                          int64_t npts, int64_t ld, int nao, double* out,
                          cudaStream_t s);
// grad (natm, 3) += scale * sum over the AOs of each atom of aodot (virtual
// shells in order)
cudaError_t launch_atom_sum(const double* aodot, const int* vs_ao0, const int* vs_nf,
                            const int* vs_atom, int nvshell, int natm, double scale,
                            double* grad, cudaStream_t s);

}  // namespace wb
