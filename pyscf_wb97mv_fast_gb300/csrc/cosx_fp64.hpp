// Plain FP64 form of the fused screen + G kernels (cosx_fp64.cu): argument
// block and launchers.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace wb {

constexpr int kBoys64Nodes = 145;   // T_k = k / 4, k = 0..144
constexpr int kBoys64Cols = 20;     // F_m(T_k), m = 0..19 (L <= 6 + 11 Taylor terms)

struct CosxF64Args {
    const double* F;            // (nao, ld) AO-major, FP64
    double* G;                  // (nao, ld) AO-major, FP64, accumulated
    const double* coords;       // (npts, 3) molecule frame
    long long ld;
    int npts;
    double omega;
    // screening inputs of the FP32 path (32-point blocks)
    const int4* khdr;
    const int2* pshell;
    const float2* ptau;
    const float4* bnd;
    const float* bpref;
    const float4* blk_cr;
    const float* blk_msh;
    int nblk;
    int nvshell;
    float tol;                  // tile_tol / 1.001, <= 0 keeps every task
    int pp_begin[10];           // first primitive pair of each class
    // FP64 pair data: per primitive pair P (3), p, folded prefactor; per
    // class the Hermite E block from e_base[c]
    const double* P;
    const double* p;
    const double* pref;
    const double* E;
    long long e_base[10];
    const double* boys;         // kBoys64Nodes x kBoys64Cols
    const double* c2s;          // l = 2 (6 x 5) at 0, l = 3 (10 x 7) at 30, row-major
    const long long* pflops;
    const int* pnint;
    unsigned long long* counters;   // per class: kept, flops, ints
    int* work;                      // per class block counter (zeroed)
};

// one class launch (classes 0..9); the f classes live in cosx_fp64_f.cu
cudaError_t launch_cosx_fp64_class(int cls, const CosxF64Args& a, int pb, int pe,
                                   int nsm, cudaStream_t s);
cudaError_t launch_cosx_fp64_f(int cls, const CosxF64Args& a, int pb, int pe,
                               int nsm, cudaStream_t s);
cudaError_t launch_weight_g64(const double* G, const double* w, int64_t npts,
                              int64_t ld, int nao, double* out, cudaStream_t s);

}  // namespace wb
