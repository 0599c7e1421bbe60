// C ABI of libwb97mv_gb300 (declarations and contracts in
// include/wb97mv_gb300.h).  Host orchestration of the COSX K build: table
// upload, workspace carving, the per-tile pipeline and cuBLAS GEMMs.
#include <cublas_v2.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <climits>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <set>
#include <string>
#include <vector>

#include "host.hpp"
#include "cosx_fp64.hpp"
#include "cosx_grad64.hpp"
#include "generated/cosx_layout.h"
#include "scf.hpp"
#include "launch.hpp"
#include "ozaki.hpp"
#include "wb97mv_gb300.h"

namespace {

thread_local std::string g_err;

int fail(int code, const std::string& msg) {
    g_err = msg;
    return code;
}

int cuda_fail(cudaError_t e, const char* where) {
    if (e == cudaErrorMemoryAllocation)
        return fail(WB_ERR_OUT_OF_MEMORY, std::string(where) + ": " +
                                              cudaGetErrorString(e));
    return fail(WB_ERR_CUDA, std::string(where) + ": " + cudaGetErrorString(e));
}

#define WB_CUDA(call)                                              \
    do {                                                           \
        cudaError_t e_ = (call);                                   \
        if (e_ != cudaSuccess) return cuda_fail(e_, #call);        \
    } while (0)

#define WB_CUBLAS(call)                                            \
    do {                                                           \
        cublasStatus_t s_ = (call);                                \
        if (s_ != CUBLAS_STATUS_SUCCESS)                           \
            return fail(s_ == CUBLAS_STATUS_ALLOC_FAILED           \
                            ? WB_ERR_OUT_OF_MEMORY : WB_ERR_CUBLAS,\
                        std::string(#call) + " failed, status " +  \
                            std::to_string((int)s_));              \
    } while (0)

inline size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

// largest dynamic shared memory per CTA for staged primitive-pair records
constexpr size_t kStageMaxBytes = 96 * 1024;
constexpr size_t kCublasWorkspace = 32u << 20;    // bytes per handle
// per-class counters (kept, flops, ints) and one status word (a record
// staging wait of a class kernel that gave up)
constexpr int kCounterWords = 3 * wb::NCLASS + 1;
// default staged classes: (0,0) (1,0) (1,1) (2,1)
constexpr long long kStageClasses = 0x1110100000LL;
// default classes with a dual-omega kernel: (0,0) (1,0) (2,0) (2,1)
constexpr long long kDualClasses = 0x1101100000LL;
inline int64_t round32(int64_t x) { return (x + 31) / 32 * 32; }

// Boys table per device, built once per process
std::mutex g_boys_mu;
std::map<int, float4*> g_boys;

int device_boys(int dev, float4** out) {
    std::lock_guard<std::mutex> lk(g_boys_mu);
    auto it = g_boys.find(dev);
    if (it != g_boys.end()) { *out = it->second; return WB_OK; }
    const std::vector<float> tab = wb::boys_table();
    float4* d = nullptr;
    WB_CUDA(cudaMalloc(&d, tab.size() * sizeof(float)));
    WB_CUDA(cudaMemcpy(d, tab.data(), tab.size() * sizeof(float),
                       cudaMemcpyHostToDevice));
    g_boys[dev] = d;
    *out = d;
    return WB_OK;
}

// the __constant__ tables (cart->sph, exp) per device, uploaded once per
// process: a handle created on one thread must not rewrite constant memory
// that another thread's kernels are reading
std::mutex g_const_mu;
std::set<int> g_const_dev;

int upload_constants() {
    int dev = 0;
    WB_CUDA(cudaGetDevice(&dev));
    std::lock_guard<std::mutex> lk(g_const_mu);
    if (g_const_dev.count(dev)) return WB_OK;
    std::vector<double> c[4];
    for (int l = 0; l < 4; ++l) c[l] = wb::cart2sph(l);
    WB_CUDA(wb::upload_c2s_tables(c[0].data(), c[1].data(), c[2].data(),
                                  c[3].data()));
    float f[4][70];
    std::memset(f, 0, sizeof(f));
    for (int l = 0; l < 4; ++l)
        for (size_t i = 0; i < c[l].size(); ++i) f[l][i] = (float)c[l][i];
    WB_CUDA(wb::upload_c2s_f(&f[0][0]));
    double t64[64];
    for (int j = 0; j < 64; ++j)
        t64[j] = (double)std::exp2l(-(long double)j / 64.0L);   // rounded once
    WB_CUDA(wb::upload_exp_table(t64));
    {
        double all[110];
        int o = 0;
        for (int l = 0; l < 4; ++l)
            for (size_t i = 0; i < c[l].size(); ++i) all[o++] = c[l][i];
        WB_CUDA(wb::scf::upload_int1e_c2s(all));
    }
    g_const_dev.insert(dev);
    return WB_OK;
}

}  // namespace

namespace wb {
void set_last_error(const std::string& msg) { g_err = msg; }
}  // namespace wb

struct wb_cosx {
    int device = 0;
    int nsm = 1;
    wb::HostPairs hp;
    cublasHandle_t cublas = nullptr;
    void* block = nullptr;
    // pair tables
    float4* geo = nullptr;
    double* p = nullptr;
    double* pref = nullptr;
    float4* E = nullptr;
    int4* hdr = nullptr;
    int4* khdr = nullptr;
    int4* gsrc = nullptr;
    int2* pshell = nullptr;
    float2* ptau = nullptr;
    float4* bnd = nullptr;
    float* bpref = nullptr;
    long long* pflops = nullptr;
    int* pnint = nullptr;
    int* vs_ao0 = nullptr;
    int* vs_nf = nullptr;
    int* pclass = nullptr;
    int* pl = nullptr;
    int* estride = nullptr;
    float4* boys = nullptr;
    // AO evaluation (physical shells)
    int nbas = 0;
    int* sh_l = nullptr;
    int* sh_np = nullptr;
    int* sh_nc = nullptr;
    int* sh_eoff = nullptr;
    int* sh_coff = nullptr;
    int* sh_ao0 = nullptr;
    double* sh_ctr = nullptr;
    double* exps = nullptr;
    double* coeffs = nullptr;
    int blocks_per_sm[wb::NCLASS][2] = {};   // [class][far variant]
    int recmax[wb::NCLASS] = {0};            // float4 of the largest task record
    size_t stage_smem[wb::NCLASS] = {0};     // dynamic smem of the staged variant
                                             // (0: register-prefetch variant)
    // dual-omega variant (two omegas per launch): record size, dynamic smem,
    // occupancy; usable when every class with pairs supports it
    int recmax2[wb::NCLASS] = {0};
    size_t stage_smem2[wb::NCLASS] = {0};
    int blocks_per_sm2[wb::NCLASS] = {0};
    bool dual_cls[wb::NCLASS] = {false};   // class runs its dual-omega kernel
    bool dual_ok = false;                  // two-omega passes are on
    // class launches run concurrently on their own streams (fork / join by
    // events on the caller's stream), largest estimated work first
    cudaStream_t cstream[wb::NCLASS] = {};
    cudaEvent_t cdone[wb::NCLASS] = {};
    cudaEvent_t fork = nullptr;
    int corder[wb::NCLASS] = {0};
    int pts[wb::NCLASS] = {0};       // points per lane of each class kernel
    int pts2[wb::NCLASS] = {0};      // the same for the dual-omega kernels
    // block order (costliest first) learnt from the previous launch on a
    // grid of the same padded size: per class, stride floats of block
    // costs and ints of order; bo_n[c] = blocks of the order held (0: none)
    float* bcost = nullptr;
    int* border = nullptr;
    int64_t bo_stride = 0, bo_ld = -1;
    int bo_n[wb::NCLASS] = {0};
    // first pair of the second half of each class's blocks (WB_COSX_SPLIT):
    // a run boundary near the middle of the class's model flops
    int split[wb::NCLASS] = {0};
    // FP64 pair data of the plain FP64 form (wb_cosx_get_k_fp64), uploaded
    // on its first call: P per primitive pair, the class E blocks, the FP64
    // Boys table followed by the FP64 c2s tables of l = 2, 3
    void* cublas_ws = nullptr;       // fixed cuBLAS workspace (kCublasWorkspace)
    double* f64_P = nullptr;
    double* f64_E = nullptr;
    double* f64_boys = nullptr;
    long long f64_ebase[wb::NCLASS] = {0};
    double* f64_alpha = nullptr;     // bra exponent per primitive pair
    double* f64_vsxyz = nullptr;     // virtual shell centres (3 each)
    int* vs_atom = nullptr;          // virtual shell atoms
    double origin[3] = {0.0, 0.0, 0.0};   // frame of the device coordinates
    // SCF helpers (wb_scf_int1e, wb_hartree), set up on first use: per pair
    // L = la + lb; per primitive pair the offset of its Hermite density and
    // p in FP32; nuclei (x, y, z, Z) in the handle frame
    int* pair_L = nullptr;
    long long* dh_off = nullptr;
    float* p32 = nullptr;
    int64_t ndh = 0;
    double* nuc = nullptr;
    int nuc_cap = 0;
};

namespace {

struct WsLayout {
    size_t om = 0, rec = 0, om2 = 0, rec2 = 0, recb = 0, gh = 0, gl = 0;
    size_t counters = 0, work = 0;
    size_t subcr[3] = {0, 0, 0}, msh[3] = {0, 0, 0};  // 32/64/128-point blocks
    size_t gcls = 0, gcls2 = 0, gclsH = 0, gcls2H = 0;
    size_t X = 0, F64 = 0, F32 = 0, G32 = 0, G32b = 0, oz = 0, total = 0;
};

WsLayout ws_layout(const wb_cosx* h, int64_t ldt, bool full) {
    WsLayout L;
    size_t off = 0;
    auto take = [&](size_t bytes) {
        const size_t o = off;
        off = align256(off + bytes);
        return o;
    };
    const int nao = h->hp.nao;
    L.counters = take(sizeof(unsigned long long) * kCounterWords);
    L.work = take(sizeof(int) * 2 * wb::NCLASS);     // per class, per omega slot
    L.om = take(sizeof(float) * wb::OMEGA_REC * (size_t)std::max(h->hp.npp, 1));
    L.rec = take(sizeof(float4) * (size_t)std::max<int64_t>(h->hp.nrec, 1));
    // second omega of a dual-omega build: its omega record, the dual
    // records and its class buffers (and G below)
    L.om2 = take(sizeof(float) * wb::OMEGA_REC * (size_t)std::max(h->hp.npp, 1));
    L.rec2 = take(sizeof(float4) * (size_t)std::max<int64_t>(h->hp.nrec2, 1));
    L.recb = take(sizeof(float4) * (size_t)std::max<int64_t>(h->hp.nrec, 1));
    L.gh = take(sizeof(float) * 3 * (size_t)ldt);
    L.gl = take(sizeof(float) * 3 * (size_t)ldt);
    for (int b = 0; b < 3; ++b) {
        const int64_t bp = 32 << b;
        const int64_t nblk = (ldt + bp - 1) / bp;
        L.subcr[b] = take(sizeof(float4) * (size_t)nblk);
        L.msh[b] = take(sizeof(float) * (size_t)nblk * std::max(h->hp.nvshell, 1));
    }
    L.gcls = take(sizeof(float) * (size_t)std::max<int64_t>(h->hp.ncrow, 1) * ldt);
    L.gcls2 = take(sizeof(float) * (size_t)std::max<int64_t>(h->hp.ncrow, 1) * ldt);
#if WB_COSX_SPLIT
    L.gclsH = take(sizeof(float) * (size_t)std::max<int64_t>(h->hp.ncrow, 1) * ldt);
    L.gcls2H = take(sizeof(float) * (size_t)std::max<int64_t>(h->hp.ncrow, 1) * ldt);
#endif
    if (full) {
        L.X = take(sizeof(double) * (size_t)nao * ldt);
        L.F32 = take(sizeof(float) * (size_t)nao * ldt);
        L.G32 = take(sizeof(float) * (size_t)nao * ldt);
        L.G32b = take(sizeof(float) * (size_t)nao * ldt);
        // scratch shared by the FP64 DGEMM path (F64 / w o G) and the
        // bf16 Ozaki path (slices, level outputs): never live together
        const size_t dg = sizeof(double) * (size_t)nao * ldt;
        const size_t oz = std::max(wb::ozaki_f_bytes(nao, ldt),
                                   wb::ozaki_k_bytes(nao, ldt, 2));
        L.F64 = take(std::max(dg, oz));
        L.oz = L.F64;
    }
    L.total = off;
    return L;
}

template<typename T>
T* at(void* base, size_t off) {
    return reinterpret_cast<T*>(static_cast<char*>(base) + off);
}

wb::CosxArgs make_args(const wb_cosx* h, void* ws, const WsLayout& L,
                       int64_t ldt, int64_t npts_t, const float* F,
                       double tile_tol) {
    wb::CosxArgs a;
    std::memset(&a, 0, sizeof(a));
    a.F = F;
    for (int c = 0; c < wb::NCLASS; ++c) {
        a.Gcls[c] = at<float>(ws, L.gcls) + h->hp.crow_base[c] * ldt;
        a.crow[c] = (int)h->hp.crow[c];
    }
    a.ld = ldt;
    a.npts = (int)npts_t;
    a.nsub = (int)(ldt / 32);
    a.geo = h->geo;
    a.om = at<float4>(ws, L.om);
    for (int c = 0; c < wb::NCLASS; ++c) {
        a.Ecls[c] = h->E + h->hp.cls[c].e_base / 4;
        a.pp_begin[c] = h->hp.cls[c].pp_begin;
        a.rec[c] = at<float4>(ws, L.rec) + h->hp.rec_off[c];
        a.recmax[c] = h->recmax[c];
        a.rec2[c] = at<float4>(ws, L.rec2) + h->hp.rec_off2[c];
        a.recmax2[c] = h->recmax2[c];
        a.Gcls2[c] = at<float>(ws, L.gcls2) + h->hp.crow_base[c] * ldt;
    }
    a.hdr = h->hdr;
    a.khdr = h->khdr;
    a.pshell = h->pshell;
    a.ptau = h->ptau;
    a.bnd = h->bnd;
    a.bpref = h->bpref;
    for (int b = 0; b < 3; ++b) {
        const int64_t bp = 32 << b;
        a.blk_cr[b] = at<float4>(ws, L.subcr[b]);
        a.blk_msh[b] = at<float>(ws, L.msh[b]);
        a.nblk[b] = (int)((ldt + bp - 1) / bp);
    }
    a.nvshell = h->hp.nvshell;
    a.tol = tile_tol > 0.0 ? (float)(tile_tol / 1.001) : 0.0f;
    if (tile_tol > 0.0 && a.tol <= 0.0f) a.tol = 1e-38f;
    a.gxyz_hi = at<float>(ws, L.gh);
    a.gxyz_lo = at<float>(ws, L.gl);
    a.boys = h->boys;
    a.pflops = h->pflops;
    a.pnint = h->pnint;
    a.counters = at<unsigned long long>(ws, L.counters);
    a.status = a.counters + 3 * wb::NCLASS;
    a.work = at<int>(ws, L.work);
    for (int c = 0; c < wb::NCLASS; ++c) {
        a.cls_pb[c] = h->hp.cls[c].pair_begin;
        a.cls_pe[c] = h->hp.cls[c].pair_end;
    }
#if WB_COSX_SPLIT
    for (int c = 0; c < wb::NCLASS; ++c) {
        a.GclsH[c] = at<float>(ws, L.gclsH) + h->hp.crow_base[c] * ldt;
        a.Gcls2H[c] = at<float>(ws, L.gcls2H) + h->hp.crow_base[c] * ldt;
        a.cls_split[c] = h->split[c];
    }
#endif
    return a;
}

// per-omega primitive-pair data: the omega record and the packed class
// records the G kernels read
int prepare_omega(wb_cosx* h, double omega, void* ws, const WsLayout& L,
                  cudaStream_t s) {
    WB_CUDA(wb::launch_omega(h->hp.npp, h->p, h->pref, omega,
                             at<float4>(ws, L.om), s));
    wb::RecPack P;
    for (int c = 0; c < wb::NCLASS; ++c) {
        P.pp_begin[c] = h->hp.cls[c].pp_begin;
        P.pp_end[c] = h->hp.cls[c].pp_end;
        P.stride[c] = wb::kRecStride[c];
        P.nom[c] = wb::kRecNom[c];
        P.ne[c] = wb::kRecNe[c];
        P.rec_off[c] = h->hp.rec_off[c];
        P.e_off[c] = h->hp.cls[c].e_base / 4;
    }
    WB_CUDA(wb::launch_pack_records(P, h->hp.npp, h->geo, at<float4>(ws, L.om),
                                    h->E, at<float4>(ws, L.rec), s));
    return WB_OK;
}

// the same for two omegas at once: both omega records and the dual-layout
// class records (slot a first)
int prepare_omega_dual(wb_cosx* h, double omega_a, double omega_b, void* ws,
                       const WsLayout& L, cudaStream_t s) {
    WB_CUDA(wb::launch_omega(h->hp.npp, h->p, h->pref, omega_a,
                             at<float4>(ws, L.om), s));
    WB_CUDA(wb::launch_omega(h->hp.npp, h->p, h->pref, omega_b,
                             at<float4>(ws, L.om2), s));
    wb::RecPack P;
    for (int c = 0; c < wb::NCLASS; ++c) {
        P.pp_begin[c] = h->hp.cls[c].pp_begin;
        P.pp_end[c] = h->hp.cls[c].pp_end;
        P.stride[c] = wb::kRecStride2[c];
        P.nom[c] = wb::kRecNom[c];
        P.ne[c] = wb::kRecNe[c];
        P.rec_off[c] = h->hp.rec_off2[c];
        P.e_off[c] = h->hp.cls[c].e_base / 4;
    }
    WB_CUDA(wb::launch_pack_records2(P, h->hp.npp, h->geo, at<float4>(ws, L.om),
                                     at<float4>(ws, L.om2), h->E,
                                     at<float4>(ws, L.rec2), s));
    // single-omega records of both slots for the classes without a dual
    // kernel
    bool singles = false;
    for (int c = 0; c < wb::NCLASS; ++c)
        singles = singles || (h->hp.cls[c].pair_end > h->hp.cls[c].pair_begin &&
                              !h->dual_cls[c]);
    if (singles) {
        for (int c = 0; c < wb::NCLASS; ++c) {
            P.stride[c] = wb::kRecStride[c];
            P.rec_off[c] = h->hp.rec_off[c];
        }
        WB_CUDA(wb::launch_pack_records(P, h->hp.npp, h->geo, at<float4>(ws, L.om),
                                        h->E, at<float4>(ws, L.rec), s));
        WB_CUDA(wb::launch_pack_records(P, h->hp.npp, h->geo, at<float4>(ws, L.om2),
                                        h->E, at<float4>(ws, L.recb), s));
    }
    return WB_OK;
}

// grid coordinates (FP32 hi / lo) and block statistics of one tile: they
// depend on the points and F only, so one pass serves every omega
int tile_prep(wb_cosx* h, const double* coords, const double* weights,
              int64_t npts_t, int64_t ldt, const float* F, void* ws,
              const WsLayout& L, cudaStream_t s, int* launches) {
    WB_CUDA(wb::launch_grid_prep(coords, npts_t, ldt, at<float>(ws, L.gh),
                                 at<float>(ws, L.gl), s));
    wb::BlockStatsOut bo;
    for (int b = 0; b < 3; ++b) {
        bo.cr[b] = at<float4>(ws, L.subcr[b]);
        bo.msh[b] = at<float>(ws, L.msh[b]);
    }
    WB_CUDA(wb::launch_sub_stats(coords, weights, F, npts_t, ldt, h->hp.nvshell,
                                 h->vs_ao0, h->vs_nf, bo, s));
    *launches += 2;
    return WB_OK;
}

#ifndef WB_COSX_BLOCK_ORDER
#define WB_COSX_BLOCK_ORDER 1
#endif

// blocks of the class kernel that runs for class c (its points per lane)
int class_nblk(const wb_cosx* h, const wb::CosxArgs& a, int c, bool dual) {
    const int pc = dual ? h->pts2[c] : h->pts[c];
    // with WB_COSX_SPLIT a block is two items
    return (WB_COSX_SPLIT ? 2 : 1) * a.nblk[pc == 4 ? 2 : pc - 1];
}

// cost / order arrays for a tile of ldt points (grown on demand; a new
// padded size drops the orders held), then the per-class pointers of a:
// every class records its block costs, and takes its blocks in the held
// order when that order covers the same blocks
int block_order_args(wb_cosx* h, int64_t ldt, wb::CosxArgs& a,
                     const bool* dual, cudaStream_t s) {
    if (!WB_COSX_BLOCK_ORDER) return WB_OK;
    const int64_t stride = (WB_COSX_SPLIT ? 2 : 1) * ((ldt + 31) / 32);
    if (stride > h->bo_stride) {
        WB_CUDA(cudaStreamSynchronize(s));
        if (h->bcost) cudaFree(h->bcost);
        if (h->border) cudaFree(h->border);
        h->bcost = nullptr;
        h->border = nullptr;
        h->bo_stride = 0;
        WB_CUDA(cudaMalloc(&h->bcost, sizeof(float) * wb::NCLASS * stride));
        WB_CUDA(cudaMalloc(&h->border, sizeof(int) * wb::NCLASS * stride));
        h->bo_stride = stride;
        h->bo_ld = -1;
    }
    if (h->bo_ld != ldt) {
        for (int c = 0; c < wb::NCLASS; ++c) h->bo_n[c] = 0;
        h->bo_ld = ldt;
    }
    for (int c = 0; c < wb::NCLASS; ++c) {
        a.bcost[c] = h->bcost + c * h->bo_stride;
        a.border[c] = h->bo_n[c] == class_nblk(h, a, c, dual[c])
                          ? h->border + c * h->bo_stride : nullptr;
    }
    return WB_OK;
}

// after the class launches: the order of the next launch from the costs
// just recorded (classes that ran)
int block_order_update(wb_cosx* h, const wb::CosxArgs& a, const bool* ran,
                       const bool* dual, cudaStream_t s, int* launches) {
    if (!WB_COSX_BLOCK_ORDER) return WB_OK;
    wb::BlockOrderArgs P;
    P.cost = h->bcost;
    P.order = h->border;
    P.stride = h->bo_stride;
    for (int c = 0; c < wb::NCLASS; ++c)
        P.n[c] = ran[c] ? class_nblk(h, a, c, dual[c]) : 0;
    WB_CUDA(wb::launch_block_order(P, s));
    for (int c = 0; c < wb::NCLASS; ++c)
        if (ran[c]) h->bo_n[c] = P.n[c];
    *launches += 1;
    return WB_OK;
}

// the class launches of one tile (after tile_prep and prepare_omega); F and
// G are (nao, ldt) AO-major.  The classes fill their own partial-G buffers
// concurrently; G is their fixed-order sum.
int run_g_classes(wb_cosx* h, int64_t npts_t, int64_t ldt, const float* F,
                  float* G, double omega, double tile_tol, void* ws,
                  const WsLayout& L, cudaStream_t s, int* launches) {
    wb::CosxArgs a = make_args(h, ws, L, ldt, npts_t, F, tile_tol);
    const bool single[wb::NCLASS] = {};
    bool ran[wb::NCLASS] = {};
    {
        const int st = block_order_args(h, ldt, a, single, s);
        if (st != WB_OK) return st;
    }
    // the far-field R000 variant pays where T = theta p r^2 >= 36 is common:
    // the full-range operator (theta = 1); long-range omegas keep T small
    const bool far = omega == 0.0;
    // (the class kernels zero their buffers block by block)
    WB_CUDA(cudaMemsetAsync(at<int>(ws, L.work), 0, sizeof(int) * wb::NCLASS, s));
    WB_CUDA(cudaEventRecord(h->fork, s));
    for (int i = 0; i < wb::NCLASS; ++i) {
        const int c = h->corder[i];
        const wb::ClassRange& r = h->hp.cls[c];
        if (r.pair_end <= r.pair_begin) continue;
        const int lvl = h->pts[c] == 4 ? 2 : h->pts[c] - 1;
        const int want = ((WB_COSX_SPLIT ? 2 : 1) * a.nblk[lvl] + 3) / 4;
        const int cap = std::max(1, h->blocks_per_sm[c][far ? 1 : 0]) * h->nsm;
        const int grid = std::max(1, std::min(want, cap));
        WB_CUDA(cudaStreamWaitEvent(h->cstream[c], h->fork, 0));
        WB_CUDA(wb::launch_cosx_class_range(c, a, r.pair_begin, r.pair_end,
                                            grid, h->cstream[c], far,
                                            h->stage_smem[c]));
        WB_CUDA(cudaEventRecord(h->cdone[c], h->cstream[c]));
        WB_CUDA(cudaStreamWaitEvent(s, h->cdone[c], 0));
        ran[c] = true;
        *launches += 1;
    }
    {
        const int st = block_order_update(h, a, ran, single, s, launches);
        if (st != WB_OK) return st;
    }
#if WB_COSX_SPLIT
    WB_CUDA(wb::launch_gsum2(at<float>(ws, L.gcls), at<float>(ws, L.gclsH), h->gsrc,
                             h->hp.nao, ldt, G, s));
#else
    WB_CUDA(wb::launch_gsum(at<float>(ws, L.gcls), h->gsrc, h->hp.nao, ldt, G, s));
#endif
    *launches += 1;
    return WB_OK;
}

// the class launches of one tile for two omegas at once (after tile_prep
// and prepare_omega_dual): slot a fills the class buffers and G_a, slot b
// the second buffers and G_b
int run_g_classes_dual(wb_cosx* h, int64_t npts_t, int64_t ldt, const float* F,
                       float* Ga, float* Gb, double omega_a, double omega_b,
                       double tile_tol, void* ws, const WsLayout& L,
                       cudaStream_t s, int* launches) {
    wb::CosxArgs a = make_args(h, ws, L, ldt, npts_t, F, tile_tol);
    bool ran[wb::NCLASS] = {};
    {
        const int st = block_order_args(h, ldt, a, h->dual_cls, s);
        if (st != WB_OK) return st;
    }
    // slot b of the single-omega kernels: its records, buffers, counters
    wb::CosxArgs b = a;
    for (int c = 0; c < wb::NCLASS; ++c) {
        b.rec[c] = at<float4>(ws, L.recb) + h->hp.rec_off[c];
        b.Gcls[c] = a.Gcls2[c];
#if WB_COSX_SPLIT
        b.GclsH[c] = a.Gcls2H[c];
#endif
    }
    b.work = a.work + wb::NCLASS;
    // (the class kernels zero their buffers block by block)
    WB_CUDA(cudaMemsetAsync(at<int>(ws, L.work), 0, sizeof(int) * 2 * wb::NCLASS, s));
    WB_CUDA(cudaEventRecord(h->fork, s));
    for (int i = 0; i < wb::NCLASS; ++i) {
        const int c = h->corder[i];
        const wb::ClassRange& r = h->hp.cls[c];
        if (r.pair_end <= r.pair_begin) continue;
        const int pc = h->dual_cls[c] ? h->pts2[c] : h->pts[c];
        const int lvl = pc == 4 ? 2 : pc - 1;
        const int want = ((WB_COSX_SPLIT ? 2 : 1) * a.nblk[lvl] + 3) / 4;
        WB_CUDA(cudaStreamWaitEvent(h->cstream[c], h->fork, 0));
        if (h->dual_cls[c]) {
            const int cap = std::max(1, h->blocks_per_sm2[c]) * h->nsm;
            WB_CUDA(wb::launch_cosx_class_range(c, a, r.pair_begin, r.pair_end,
                                                std::max(1, std::min(want, cap)),
                                                h->cstream[c], false,
                                                h->stage_smem2[c], true));
            *launches += 1;
        } else {
            const double om[2] = {omega_a, omega_b};
            for (int w = 0; w < 2; ++w) {
                const bool far = om[w] == 0.0;
                const int cap = std::max(1, h->blocks_per_sm[c][far ? 1 : 0]) * h->nsm;
                WB_CUDA(wb::launch_cosx_class_range(c, w ? b : a, r.pair_begin,
                                                    r.pair_end,
                                                    std::max(1, std::min(want, cap)),
                                                    h->cstream[c], far,
                                                    h->stage_smem[c]));
                *launches += 1;
            }
        }
        WB_CUDA(cudaEventRecord(h->cdone[c], h->cstream[c]));
        WB_CUDA(cudaStreamWaitEvent(s, h->cdone[c], 0));
        ran[c] = true;
    }
    {
        const int st = block_order_update(h, a, ran, h->dual_cls, s, launches);
        if (st != WB_OK) return st;
    }
#if WB_COSX_SPLIT
    WB_CUDA(wb::launch_gsum2(at<float>(ws, L.gcls), at<float>(ws, L.gclsH), h->gsrc,
                             h->hp.nao, ldt, Ga, s));
    WB_CUDA(wb::launch_gsum2(at<float>(ws, L.gcls2), at<float>(ws, L.gcls2H), h->gsrc,
                             h->hp.nao, ldt, Gb, s));
#else
    WB_CUDA(wb::launch_gsum(at<float>(ws, L.gcls), h->gsrc, h->hp.nao, ldt, Ga, s));
    WB_CUDA(wb::launch_gsum(at<float>(ws, L.gcls2), h->gsrc, h->hp.nao, ldt, Gb, s));
#endif
    *launches += 2;
    return WB_OK;
}

int read_stats(wb_cosx* h, void* ws, const WsLayout& L, int64_t ntasks_total,
               cudaStream_t s, wb_cosx_stats* stats, int launches) {
    if (!stats) return WB_OK;
    unsigned long long c[kCounterWords];
    WB_CUDA(cudaMemcpyAsync(c, at<unsigned long long>(ws, L.counters),
                            sizeof(c), cudaMemcpyDeviceToHost, s));
    WB_CUDA(cudaStreamSynchronize(s));
    if (c[3 * wb::NCLASS])
        return fail(WB_ERR_CUDA, "a class kernel's record staging timed out");
    std::memset(stats, 0, sizeof(*stats));
    stats->tasks_total = ntasks_total;
    for (int k = 0; k < wb::NCLASS; ++k) {
        stats->tasks_kept += (int64_t)c[3 * k];
        stats->tasks_kept_class[k] = (int64_t)c[3 * k];
        stats->model_flops += (double)c[3 * k + 1];
        stats->model_flops_class[k] = (double)c[3 * k + 1];
        stats->integrals += (double)c[3 * k + 2];
    }
    stats->kernel_launches = launches;
    (void)h;
    return WB_OK;
}

// FP64 pair data, FP64 Boys table and the FP64 c2s constants of the plain
// FP64 form, built and uploaded on its first call (synchronous copies)
int ensure_fp64(wb_cosx* h) {
    if (h->f64_P) return WB_OK;
    wb::HostPairs64 hp64;
    wb::build_pairs64(h->hp, hp64);
    std::vector<double> tab((size_t)wb::kBoys64Nodes * wb::kBoys64Cols);
    for (int k = 0; k < wb::kBoys64Nodes; ++k)
        wb::boys_f64(wb::kBoys64Cols - 1, 0.25 * k,
                     tab.data() + (size_t)k * wb::kBoys64Cols);
    // the FP64 c2s tables after the Boys table: l = 2 (6 x 5), l = 3 (10 x 7)
    const std::vector<double> d = wb::cart2sph(2), f = wb::cart2sph(3);
    tab.insert(tab.end(), d.begin(), d.end());
    tab.insert(tab.end(), f.begin(), f.end());
    double *P = nullptr, *E = nullptr, *B = nullptr;
    auto upload = [](double** dst, const std::vector<double>& v) -> cudaError_t {
        cudaError_t e = cudaMalloc(dst, sizeof(double) * std::max<size_t>(v.size(), 1));
        if (e != cudaSuccess) return e;
        if (v.empty()) return cudaSuccess;
        return cudaMemcpy(*dst, v.data(), sizeof(double) * v.size(),
                          cudaMemcpyHostToDevice);
    };
    cudaError_t e = upload(&P, hp64.P);
    if (e == cudaSuccess) e = upload(&E, hp64.E);
    if (e == cudaSuccess) e = upload(&B, tab);
    if (e != cudaSuccess) {
        if (P) cudaFree(P);
        if (E) cudaFree(E);
        if (B) cudaFree(B);
        return cuda_fail(e, "FP64 pair tables");
    }
    std::vector<double> vxyz;
    std::vector<int> vat;
    for (const wb::VShell& v : h->hp.vsh) {
        for (int x = 0; x < 3; ++x) vxyz.push_back(v.A[x]);
        vat.push_back(v.atom);
    }
    double *AL = nullptr, *VX = nullptr;
    int* VA = nullptr;
    e = upload(&AL, hp64.alpha);
    if (e == cudaSuccess) e = upload(&VX, vxyz);
    if (e == cudaSuccess) e = cudaMalloc(&VA, sizeof(int) * std::max<size_t>(vat.size(), 1));
    if (e == cudaSuccess && !vat.empty())
        e = cudaMemcpy(VA, vat.data(), sizeof(int) * vat.size(), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
        for (void* q : {(void*)P, (void*)E, (void*)B, (void*)AL, (void*)VX, (void*)VA})
            if (q) cudaFree(q);
        return cuda_fail(e, "FP64 pair tables");
    }
    h->f64_P = P;
    h->f64_E = E;
    h->f64_boys = B;
    h->f64_alpha = AL;
    h->f64_vsxyz = VX;
    h->vs_atom = VA;
    for (int c = 0; c < wb::NCLASS; ++c) h->f64_ebase[c] = hp64.e_base[c];
    return WB_OK;
}

// Hermite-density entries of one primitive pair of total angular momentum
// l, padded to a multiple of 4: every pair's block starts 16-byte aligned
// (FP32) and 32-byte aligned (FP64), so the kernel reads it with vector
// loads (the padding entries are read and never used)
inline int64_t hartree_nr_padded(int l) {
    return ((int64_t)(l + 1) * (l + 2) * (l + 3) / 6 + 3) & ~(int64_t)3;
}

// per-pair L, per-primitive-pair Hermite-density offsets and FP32 p of
// the Hartree potential (first wb_hartree call on the handle)
int ensure_hartree(wb_cosx* h) {
    if (h->pair_L) return WB_OK;
    const wb::HostPairs& hp = h->hp;
    std::vector<int> L((size_t)std::max(hp.npairs, 1), 0);
    std::vector<long long> off((size_t)std::max(hp.npp, 1), 0);
    std::vector<float> p32((size_t)std::max(hp.npp, 1), 0.0f);
    long long tot = 0;
    for (int k = 0; k < hp.npairs; ++k) {
        const int l = hp.vsh[hp.pshell[2 * k]].l + hp.vsh[hp.pshell[2 * k + 1]].l;
        L[k] = l;
        const int pp0 = hp.hdr[4 * k + 2], npp = hp.hdr[4 * k + 3] & 0xffff;
        for (int m = pp0; m < pp0 + npp; ++m) {
            off[m] = tot;
            tot += hartree_nr_padded(l);
        }
    }
    for (int m = 0; m < hp.npp; ++m) p32[m] = (float)hp.p[m];
    int* dL = nullptr;
    long long* dO = nullptr;
    float* dP = nullptr;
    cudaError_t e = cudaMalloc(&dL, sizeof(int) * L.size());
    if (e == cudaSuccess) e = cudaMalloc(&dO, sizeof(long long) * off.size());
    if (e == cudaSuccess) e = cudaMalloc(&dP, sizeof(float) * p32.size());
    if (e == cudaSuccess)
        e = cudaMemcpy(dL, L.data(), sizeof(int) * L.size(), cudaMemcpyHostToDevice);
    if (e == cudaSuccess)
        e = cudaMemcpy(dO, off.data(), sizeof(long long) * off.size(), cudaMemcpyHostToDevice);
    if (e == cudaSuccess)
        e = cudaMemcpy(dP, p32.data(), sizeof(float) * p32.size(), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
        for (void* q : {(void*)dL, (void*)dO, (void*)dP})
            if (q) cudaFree(q);
        return cuda_fail(e, "Hartree pair tables");
    }
    h->pair_L = dL;
    h->dh_off = dO;
    h->p32 = dP;
    h->ndh = std::max<long long>(tot, 1);
    return WB_OK;
}

struct HartreeLayout {
    size_t counters = 0, cr = 0, dabs = 0, dh64 = 0, dh32 = 0, total = 0;
};

HartreeLayout hartree_layout(const wb_cosx* h, int64_t npts, int64_t ndh) {
    HartreeLayout L;
    size_t off = 0;
    auto take = [&](size_t bytes) {
        const size_t o = off;
        off = align256(off + bytes);
        return o;
    };
    const int64_t nblk = (npts + 31) / 32;
    L.counters = take(256);
    L.cr = take(sizeof(float4) * (size_t)std::max<int64_t>(nblk, 1));
    L.dabs = take(sizeof(float) * (size_t)std::max(h->hp.npairs, 1));
    L.dh64 = take(sizeof(double) * (size_t)ndh);
    L.dh32 = take(sizeof(float) * (size_t)ndh);
    L.total = off;
    return L;
}

int64_t hartree_ndh(const wb::HostPairs& hp) {
    int64_t tot = 0;
    for (int k = 0; k < hp.npairs; ++k) {
        const int l = hp.vsh[hp.pshell[2 * k]].l + hp.vsh[hp.pshell[2 * k + 1]].l;
        tot += (int64_t)(hp.hdr[4 * k + 3] & 0xffff) * hartree_nr_padded(l);
    }
    return std::max<int64_t>(tot, 1);
}

struct WsLayout64 {
    WsLayout base;                  // counters, work, block statistics
    size_t X = 0, F64 = 0, F32 = 0, G64 = 0, WG = 0, total = 0;
};

WsLayout64 ws_layout_fp64(const wb_cosx* h, int64_t ld) {
    WsLayout64 L;
    size_t off = 0;
    auto take = [&](size_t bytes) {
        const size_t o = off;
        off = align256(off + bytes);
        return o;
    };
    L.base.counters = take(sizeof(unsigned long long) * kCounterWords);
    L.base.work = take(sizeof(int) * 2 * wb::NCLASS);
    for (int b = 0; b < 3; ++b) {
        const int64_t bp = 32 << b;
        const int64_t nblk = (ld + bp - 1) / bp;
        L.base.subcr[b] = take(sizeof(float4) * (size_t)nblk);
        L.base.msh[b] = take(sizeof(float) * (size_t)nblk * std::max(h->hp.nvshell, 1));
    }
    const size_t n = (size_t)h->hp.nao * ld;
    L.X = take(sizeof(double) * n);
    L.F64 = take(sizeof(double) * n);
    L.F32 = take(sizeof(float) * n);
    L.G64 = take(sizeof(double) * n);
    L.WG = take(sizeof(double) * n);
    L.total = off;
    return L;
}

}  // namespace

// -- batched K builds: several molecules, one launch per class -------------

struct wb_cosx_batch {
    int nmol = 0;
    int nom = 0;                        // omegas: 1, or 2 (slot a <= slot b)
    double om[2] = {0.0, 0.0};
    int kidx[2] = {0, 1};               // k_out matrix of slot a / b
    double tol = 0.0;
    int gemm = WB_K_GEMM_OZAKI_BF16;
    std::vector<wb_cosx*> h;
    std::vector<const double*> coords, weights;
    std::vector<int64_t> npts, ld;
    std::vector<void*> ws;
    std::vector<WsLayout> L;
    void* scratch = nullptr;            // the F / K split scratch, shared
    bool has[wb::NCLASS] = {};          // some molecule has pairs of the class
    bool dual[wb::NCLASS] = {};         // the two-omega kernel, every molecule
    size_t smem[wb::NCLASS] = {};       // staged single-omega kernel (0: prefetch)
    size_t smem2[wb::NCLASS] = {};
    int rmax[wb::NCLASS] = {}, rmax2[wb::NCLASS] = {};
    int items[wb::NCLASS] = {};         // blocks of the class over the molecules
    int order[wb::NCLASS] = {};
    void* block = nullptr;              // device: args (2 nmol), offsets, counters,
                                        // item costs and orders
    wb::CosxArgs* d_args = nullptr;
    int* d_off = nullptr;               // NCLASS x (nmol + 1)
    int* d_work = nullptr;              // NCLASS x 2
    float* d_cost = nullptr;            // NCLASS x stride: model flops per item
    int* d_order = nullptr;             // NCLASS x stride: costliest first
    int64_t stride = 0;
    bool ordered = false;               // the orders hold a previous run's costs
};

static int batch_fail(wb_cosx_batch* b, int code) {
    wb_cosx_batch_destroy(b);
    return code;
}

extern "C" {

int wb_version(void) { return 1; }

const char* wb_last_error(void) { return g_err.c_str(); }

const char* wb_status_string(int status) {
    switch (status) {
    case WB_OK: return "ok";
    case WB_ERR_INVALID_ARGUMENT: return "invalid argument";
    case WB_ERR_UNSUPPORTED: return "unsupported input";
    case WB_ERR_CUDA: return "CUDA error";
    case WB_ERR_CUBLAS: return "cuBLAS error";
    case WB_ERR_OUT_OF_MEMORY: return "out of device memory";
    case WB_ERR_WORKSPACE: return "workspace too small";
    case WB_ERR_NO_DEVICE: return "no CUDA device";
    default: return "unknown status";
    }
}

int wb_boys_f64_host(int nmax, double t, double* out) {
    if (nmax < 0 || nmax > 40 || !out || !(t >= 0.0))
        return fail(WB_ERR_INVALID_ARGUMENT, "wb_boys_f64_host: bad arguments");
    wb::boys_f64(nmax, t, out);
    return WB_OK;
}

int wb_model_flops_per_point(const wb_basis* basis, double pair_cutoff,
                             double* flops_out, int64_t* npairs_out) {
    if (!basis || !flops_out || !(pair_cutoff >= 0.0))
        return fail(WB_ERR_INVALID_ARGUMENT, "wb_model_flops_per_point: bad arguments");
    wb::HostPairs hp;
    std::string err;
    const double origin[3] = {0.0, 0.0, 0.0};
    const int st = wb::build_pairs(*basis, origin, pair_cutoff, hp, err);
    if (st != WB_OK) return fail(st, err);
    double sum = 0.0;
    for (const int64_t f : hp.pflops) sum += (double)f;
    *flops_out = sum;
    if (npairs_out) *npairs_out = hp.npairs;
    return WB_OK;
}

int wb_becke_partition(const double* points, int64_t n, const int* owner,
                       const double* atom_coords, int natm, double* out) {
    if (n < 0 || natm <= 0 || (!points && n) || (!owner && n) || !atom_coords ||
        (!out && n))
        return fail(WB_ERR_INVALID_ARGUMENT, "wb_becke_partition: bad arguments");
    for (int64_t i = 0; i < n; ++i)
        if (owner[i] < 0 || owner[i] >= natm)
            return fail(WB_ERR_INVALID_ARGUMENT, "wb_becke_partition: bad owner");
    wb::becke_partition(points, n, owner, atom_coords, natm, out);
    return WB_OK;
}

int wb_cosx_create(const wb_basis* basis, const double origin[3],
                   double pair_cutoff, wb_cosx** out) {
    if (!basis || !origin || !out)
        return fail(WB_ERR_INVALID_ARGUMENT, "wb_cosx_create: null argument");
    *out = nullptr;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev < 1) {
        cudaGetLastError();
        return fail(WB_ERR_NO_DEVICE, "wb_cosx_create: no CUDA device");
    }
    wb_cosx* h = new wb_cosx();
    std::string err;
    int st = wb::build_pairs(*basis, origin, pair_cutoff, h->hp, err);
    if (st != WB_OK) {
        delete h;
        return fail(st, err);
    }
    auto cleanup = [&](int code) {
        wb_cosx_destroy(h);
        return code;
    };
    for (int x = 0; x < 3; ++x) h->origin[x] = origin[x];
    if (cudaGetDevice(&h->device) != cudaSuccess) return cleanup(cuda_fail(cudaGetLastError(), "cudaGetDevice"));
    cudaDeviceGetAttribute(&h->nsm, cudaDevAttrMultiProcessorCount, h->device);
    if ((st = upload_constants()) != WB_OK) return cleanup(st);
    if ((st = device_boys(h->device, &h->boys)) != WB_OK) return cleanup(st);

    const wb::HostPairs& hp = h->hp;
    // physical shell tables for the AO evaluation
    h->nbas = basis->nbas;
    std::vector<int> sh_ao0(basis->nbas);
    {
        int ao = 0;
        for (int s = 0; s < basis->nbas; ++s) {
            sh_ao0[s] = ao;
            ao += basis->shell_nctr[s] * (2 * basis->shell_l[s] + 1);
        }
    }
    int nexp = 0, ncoef = 0;
    for (int s = 0; s < basis->nbas; ++s) {
        nexp = std::max(nexp, basis->shell_exp_off[s] + basis->shell_nprim[s]);
        ncoef = std::max(ncoef, basis->shell_coef_off[s] +
                                    basis->shell_nprim[s] * basis->shell_nctr[s]);
    }
    std::vector<double> ctr(3 * (size_t)std::max(basis->nbas, 1));
    for (int s = 0; s < basis->nbas; ++s)
        for (int x = 0; x < 3; ++x)
            ctr[3 * s + x] = basis->atom_coords[basis->shell_atom[s] * 3 + x] - origin[x];
    std::vector<int> pl, estr(wb::NCLASS);
    for (int k = 0; k < hp.npairs; ++k) {
        pl.push_back(hp.vsh[hp.pshell[2 * k]].l);
        pl.push_back(hp.vsh[hp.pshell[2 * k + 1]].l);
    }
    for (int la = 0; la <= 3; ++la)
        for (int lb = 0; lb <= la; ++lb) estr[wb::class_of(la, lb)] = wb::e_stride(la, lb);

    struct Piece { void** dst; const void* src; size_t bytes; };
    std::vector<Piece> pieces;
    auto add = [&](void** dst, const void* src, size_t bytes) {
        pieces.push_back({dst, src, bytes});
    };
    add((void**)&h->geo, hp.geo.data(), hp.geo.size() * sizeof(float));
    add((void**)&h->p, hp.p.data(), hp.p.size() * sizeof(double));
    add((void**)&h->pref, hp.pref.data(), hp.pref.size() * sizeof(double));
    add((void**)&h->E, hp.E.data(), hp.E.size() * sizeof(float));
    add((void**)&h->hdr, hp.hdr.data(), hp.hdr.size() * sizeof(int32_t));
    add((void**)&h->khdr, hp.khdr.data(), hp.khdr.size() * sizeof(int32_t));
    add((void**)&h->gsrc, hp.gsrc.data(), hp.gsrc.size() * sizeof(int32_t));
    add((void**)&h->pshell, hp.pshell.data(), hp.pshell.size() * sizeof(int32_t));
    add((void**)&h->ptau, hp.ptau.data(), hp.ptau.size() * sizeof(float));
    add((void**)&h->bnd, hp.bnd.data(), hp.bnd.size() * sizeof(float));
    add((void**)&h->bpref, hp.bpref.data(), hp.bpref.size() * sizeof(float));
    add((void**)&h->pflops, hp.pflops.data(), hp.pflops.size() * sizeof(int64_t));
    add((void**)&h->pnint, hp.pnint.data(), hp.pnint.size() * sizeof(int32_t));
    add((void**)&h->vs_ao0, hp.vs_ao0.data(), hp.vs_ao0.size() * sizeof(int32_t));
    add((void**)&h->vs_nf, hp.vs_nf.data(), hp.vs_nf.size() * sizeof(int32_t));
    add((void**)&h->pclass, hp.pclass.data(), hp.pclass.size() * sizeof(int32_t));
    add((void**)&h->pl, pl.data(), pl.size() * sizeof(int));
    add((void**)&h->estride, estr.data(), estr.size() * sizeof(int));
    add((void**)&h->sh_l, basis->shell_l, sizeof(int) * basis->nbas);
    add((void**)&h->sh_np, basis->shell_nprim, sizeof(int) * basis->nbas);
    add((void**)&h->sh_nc, basis->shell_nctr, sizeof(int) * basis->nbas);
    add((void**)&h->sh_eoff, basis->shell_exp_off, sizeof(int) * basis->nbas);
    add((void**)&h->sh_coff, basis->shell_coef_off, sizeof(int) * basis->nbas);
    add((void**)&h->sh_ao0, sh_ao0.data(), sizeof(int) * basis->nbas);
    add((void**)&h->sh_ctr, ctr.data(), sizeof(double) * 3 * basis->nbas);
    add((void**)&h->exps, basis->exps, sizeof(double) * nexp);
    add((void**)&h->coeffs, basis->coeffs, sizeof(double) * ncoef);
    size_t total = 0;
    for (const Piece& pc : pieces) total = align256(total + pc.bytes);
    total = std::max<size_t>(total, 256);
    cudaError_t e = cudaMalloc(&h->block, total);
    if (e != cudaSuccess) return cleanup(cuda_fail(e, "cudaMalloc(pair tables)"));
    size_t off = 0;
    for (const Piece& pc : pieces) {
        char* dst = static_cast<char*>(h->block) + off;
        *pc.dst = dst;
        if (pc.bytes) {
            e = cudaMemcpy(dst, pc.src, pc.bytes, cudaMemcpyHostToDevice);
            if (e != cudaSuccess) return cleanup(cuda_fail(e, "cudaMemcpy(pair tables)"));
        }
        off = align256(off + pc.bytes);
    }
    if (cublasCreate(&h->cublas) != CUBLAS_STATUS_SUCCESS)
        return cleanup(fail(WB_ERR_CUBLAS, "cublasCreate failed"));
    // a fixed cuBLAS workspace owned by the handle: no cuBLAS call of a
    // build allocates, so a build can be captured in a CUDA graph
    {
        const cudaError_t we = cudaMalloc(&h->cublas_ws, kCublasWorkspace);
        if (we != cudaSuccess) return cleanup(cuda_fail(we, "cuBLAS workspace"));
        if (cublasSetWorkspace(h->cublas, h->cublas_ws, kCublasWorkspace) !=
            CUBLAS_STATUS_SUCCESS)
            return cleanup(fail(WB_ERR_CUBLAS, "cublasSetWorkspace failed"));
    }
    // classes whose records are staged in shared memory: one hex digit per
    // class in class order (measured per class on the water27 workload:
    // staging wins where the register-carried record cost moves and
    // uniform-register traffic, loses where it raises spills); the
    // environment variable WB_COSX_STAGE (same digits) overrides it
    long long stage_mask = kStageClasses;
    if (const char* env = std::getenv("WB_COSX_STAGE"))
        stage_mask = std::strtoll(env, nullptr, 16);
    for (int c = 0; c < wb::NCLASS; ++c) {
        // primitive-pair records staged in shared memory (two buffers per
        // warp of the largest task's record) for the classes of the mask,
        // unless that needs more than kStageMaxBytes per CTA
        int rm = 0;
        for (int k = hp.cls[c].pair_begin; k < hp.cls[c].pair_end; ++k)
            rm = std::max(rm, (hp.hdr[4 * k + 3] & 0xffff) * wb::kRecStride[c]);
        h->recmax[c] = rm;
        const size_t smem = (size_t)(128 / 32) * 2 * rm * sizeof(float4);
        const bool stage_on = ((stage_mask >> (4 * (wb::NCLASS - 1 - c))) & 15) != 0;
        h->stage_smem[c] = (stage_on && rm > 0 && smem <= kStageMaxBytes) ? smem : 0;
        int n[2];
        for (int f = 0; f < 2; ++f)
            n[f] = wb::cosx_class_blocks_per_sm(c, f == 1, h->stage_smem[c]);
        if (h->stage_smem[c] && (n[0] == 0 || n[1] == 0)) {
            h->stage_smem[c] = 0;
            for (int f = 0; f < 2; ++f)
                n[f] = wb::cosx_class_blocks_per_sm(c, f == 1, 0);
        }
        for (int f = 0; f < 2; ++f) h->blocks_per_sm[c][f] = std::max(n[f], 1);
        // dual-omega variant: always staged, dual record layout
        int rm2 = 0;
        for (int k = hp.cls[c].pair_begin; k < hp.cls[c].pair_end; ++k)
            rm2 = std::max(rm2, (hp.hdr[4 * k + 3] & 0xffff) * wb::kRecStride2[c]);
        h->recmax2[c] = rm2;
        const size_t smem2 = (size_t)(128 / 32) * 2 * rm2 * sizeof(float4);
        if (rm2 > 0 && smem2 <= kStageMaxBytes) {
            h->stage_smem2[c] = smem2;
            h->blocks_per_sm2[c] = wb::cosx_class_blocks_per_sm(c, false, smem2, true);
        }
        h->pts[c] = wb::cosx_class_pts(c);
        h->pts2[c] = wb::cosx_class_pts(c, true);
    }
    {
        // classes that run the dual-omega kernel in a two-omega pass (one
        // hex digit per class, measured per class on the water27 workload:
        // fused wins where the shared per-task work dominates, loses where
        // two sets of accumulators spill); the others run their single-omega
        // kernel twice in the same pass.  WB_COSX_DUAL overrides the digits
        // (0 turns two-omega passes off).
        long long mask = kDualClasses;
        h->dual_ok = true;
        if (const char* env = std::getenv("WB_COSX_DUAL")) {
            mask = std::strtoll(env, nullptr, 16);
            h->dual_ok = mask != 0;
        }
        for (int c = 0; c < wb::NCLASS; ++c)
            h->dual_cls[c] = ((mask >> (4 * (wb::NCLASS - 1 - c))) & 15) != 0 &&
                             h->blocks_per_sm2[c] >= 1;
    }
    for (int c = 0; c < wb::NCLASS; ++c) {
        // the split pair of each class: past half of its model flops, moved
        // on to the next run boundary (a bra shell's run stays in one half,
        // so its G_A rows have one writer)
        const int pb = hp.cls[c].pair_begin, pe = hp.cls[c].pair_end;
        double tot = 0.0, acc = 0.0;
        for (int k = pb; k < pe; ++k) tot += (double)hp.pflops[k];
        int k = pb;
        while (k < pe && acc + (double)hp.pflops[k] <= 0.5 * tot) acc += (double)hp.pflops[k++];
        while (k > pb && k < pe && hp.pshell[2 * k] == hp.pshell[2 * (k - 1)]) ++k;
        h->split[c] = k;
    }
    {   // launch order: model flops of all pairs of a class, descending
        double work[wb::NCLASS] = {0};
        for (int c = 0; c < wb::NCLASS; ++c) {
            h->corder[c] = c;
            for (int k = hp.cls[c].pair_begin; k < hp.cls[c].pair_end; ++k)
                work[c] += (double)hp.pflops[k];
        }
        std::stable_sort(h->corder, h->corder + wb::NCLASS,
                         [&](int x, int y) { return work[x] > work[y]; });
    }
    for (int c = 0; c < wb::NCLASS; ++c) {
        e = cudaStreamCreateWithFlags(&h->cstream[c], cudaStreamNonBlocking);
        if (e == cudaSuccess)
            e = cudaEventCreateWithFlags(&h->cdone[c], cudaEventDisableTiming);
        if (e != cudaSuccess) return cleanup(cuda_fail(e, "class streams"));
    }
    e = cudaEventCreateWithFlags(&h->fork, cudaEventDisableTiming);
    if (e != cudaSuccess) return cleanup(cuda_fail(e, "class streams"));
    *out = h;
    return WB_OK;
}

int wb_cosx_destroy(wb_cosx* h) {
    if (!h) return WB_OK;
    if (h->cublas) cublasDestroy(h->cublas);
    for (int c = 0; c < wb::NCLASS; ++c) {
        if (h->cstream[c]) cudaStreamDestroy(h->cstream[c]);
        if (h->cdone[c]) cudaEventDestroy(h->cdone[c]);
    }
    if (h->fork) cudaEventDestroy(h->fork);
    if (h->block) cudaFree(h->block);
    if (h->bcost) cudaFree(h->bcost);
    if (h->border) cudaFree(h->border);
    if (h->cublas_ws) cudaFree(h->cublas_ws);
    if (h->f64_P) cudaFree(h->f64_P);
    if (h->f64_E) cudaFree(h->f64_E);
    if (h->f64_boys) cudaFree(h->f64_boys);
    if (h->f64_alpha) cudaFree(h->f64_alpha);
    if (h->f64_vsxyz) cudaFree(h->f64_vsxyz);
    if (h->vs_atom) cudaFree(h->vs_atom);
    for (void* q : {(void*)h->pair_L, (void*)h->dh_off, (void*)h->p32, (void*)h->nuc})
        if (q) cudaFree(q);
    delete h;
    return WB_OK;
}

int wb_cosx_get_info(const wb_cosx* h, wb_cosx_info* info) {
    if (!h || !info) return fail(WB_ERR_INVALID_ARGUMENT, "wb_cosx_get_info: null");
    std::memset(info, 0, sizeof(*info));
    info->nao = h->hp.nao;
    info->nbas = h->hp.nvshell;
    info->npairs = h->hp.npairs;
    info->nprim_pairs = h->hp.npp;
    for (int c = 0; c < wb::NCLASS; ++c) {
        info->class_pairs[c] = h->hp.cls[c].pair_end - h->hp.cls[c].pair_begin;
        info->class_prim_pairs[c] = h->hp.cls[c].pp_end - h->hp.cls[c].pp_begin;
    }
    return WB_OK;
}

int64_t wb_cosx_export_pairs(const wb_cosx* h, int64_t* rows, int64_t cap) {
    if (!h) return 0;
    const wb::HostPairs& hp = h->hp;
    int64_t n = std::min<int64_t>(cap, hp.npairs);
    for (int64_t k = 0; k < n && rows; ++k) {
        int64_t* r = rows + 8 * k;
        r[0] = hp.hdr[4 * k]; r[1] = hp.hdr[4 * k + 1]; r[2] = hp.hdr[4 * k + 2];
        r[3] = hp.hdr[4 * k + 3]; r[4] = hp.pclass[k]; r[5] = hp.pish[k];
        r[6] = hp.pjsh[k]; r[7] = hp.pflops[k];
    }
    return rows ? n : hp.npairs;
}

size_t wb_cosx_workspace_bytes(const wb_cosx* h, int64_t npts,
                               int64_t tile_pts) {
    if (!h || npts < 0) return 0;
    int64_t t = tile_pts > 0 ? std::min(round32(tile_pts), round32(npts)) : round32(npts);
    t = std::max<int64_t>(t, 32);
    return ws_layout(h, t, true).total;
}

int wb_cosx_get_k(wb_cosx* h, const double* coords, const double* weights,
                  int64_t npts, const double* qd, double omega,
                  double tile_tol, int64_t tile_pts, int flags, double* k_out,
                  void* workspace, size_t workspace_bytes, void* stream,
                  wb_cosx_stats* stats) {
    return wb_cosx_get_k_multi(h, coords, weights, npts, qd, 1, &omega,
                               tile_tol, tile_pts, flags, k_out, workspace,
                               workspace_bytes, stream, stats);
}

int wb_cosx_get_k_multi(wb_cosx* h, const double* coords,
                        const double* weights, int64_t npts, const double* qd,
                        int nomega, const double* omegas, double tile_tol,
                        int64_t tile_pts, int flags, double* k_out,
                        void* workspace, size_t workspace_bytes, void* stream,
                        wb_cosx_stats* stats) {
    if (!h || !k_out || !qd || npts < 0 || (npts && (!coords || !weights)) ||
        nomega < 1 || !omegas)
        return fail(WB_ERR_INVALID_ARGUMENT, "wb_cosx_get_k: bad arguments");
    for (int j = 0; j < nomega; ++j)
        if (!(omegas[j] >= 0.0))
            return fail(WB_ERR_INVALID_ARGUMENT, "wb_cosx_get_k: omega must be >= 0");
    if (!(tile_tol >= 0.0))
        return fail(WB_ERR_INVALID_ARGUMENT, "wb_cosx_get_k: tile_tol must be >= 0");
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const int nao = h->hp.nao;
    const size_t kk = (size_t)nao * nao;
    int64_t tile = tile_pts > 0 ? round32(tile_pts) : round32(std::max<int64_t>(npts, 1));
    tile = std::max<int64_t>(std::min(tile, round32(std::max<int64_t>(npts, 1))), 32);
    if (tile > INT32_MAX - 64)
        return fail(WB_ERR_UNSUPPORTED, "wb_cosx_get_k: tile above 2^31 points");
    const WsLayout L = ws_layout(h, tile, true);
    if (!workspace || workspace_bytes < L.total)
        return fail(WB_ERR_WORKSPACE, "wb_cosx_get_k: workspace needs " +
                                          std::to_string(L.total) + " bytes");
    WB_CUBLAS(cublasSetStream(h->cublas, s));
    const int gemm_mode = flags & 3;
    const bool oz_f = gemm_mode == WB_K_GEMM_OZAKI_BF16 && wb::ozaki_f_supported(nao);
    const bool oz_k = gemm_mode == WB_K_GEMM_OZAKI_BF16;
    if (gemm_mode == WB_K_GEMM_EMULATED_FP64) {
        WB_CUBLAS(cublasSetMathMode(h->cublas, CUBLAS_FP64_EMULATED_FIXEDPOINT_MATH));
        WB_CUBLAS(cublasSetEmulationStrategy(h->cublas, CUBLAS_EMULATION_STRATEGY_EAGER));
    } else {
        WB_CUBLAS(cublasSetMathMode(h->cublas, CUBLAS_DEFAULT_MATH));
    }
    WB_CUDA(cudaMemsetAsync(at<void>(workspace, L.counters), 0,
                            sizeof(unsigned long long) * kCounterWords, s));
    int launches = 1;
    if (npts == 0) {
        WB_CUDA(cudaMemsetAsync(k_out, 0, sizeof(double) * kk * nomega, s));
        return read_stats(h, workspace, L, 0, s, stats, launches);
    }
    double* X = at<double>(workspace, L.X);
    double* F64 = at<double>(workspace, L.F64);
    float* F32 = at<float>(workspace, L.F32);
    float* G32 = at<float>(workspace, L.G32);
    float* G32b = at<float>(workspace, L.G32b);
    int64_t ntasks = 0;
    const double one = 1.0, zero = 0.0;
    const bool prof = (flags & WB_K_PROFILE) && stats;
    // phase events: AO, F GEMM, F cast, tile prep + per omega (omega data,
    // G, weight, K GEMM)
    cudaEvent_t ev[2] = {};
    double phase[6] = {0, 0, 0, 0, 0, 0};
    if (prof)
        for (int i = 0; i < 2; ++i) WB_CUDA(cudaEventCreate(&ev[i]));
    int cur = 0;
    auto mark = [&]() -> int {
        // closes the running phase `cur` (timed from the last mark)
        if (!prof) return WB_OK;
        WB_CUDA(cudaEventRecord(ev[1], s));
        WB_CUDA(cudaEventSynchronize(ev[1]));
        float ms = 0.0f;
        WB_CUDA(cudaEventElapsedTime(&ms, ev[0], ev[1]));
        phase[cur] += ms;
        WB_CUDA(cudaEventRecord(ev[0], s));
        return WB_OK;
    };
    auto phase_to = [&](int p) -> int {
        const int st = mark();
        cur = p;
        return st;
    };
    if (prof) WB_CUDA(cudaEventRecord(ev[0], s));
    int st = WB_OK;
    for (int64_t i0 = 0; i0 < npts; i0 += tile) {
        const int64_t nt = std::min(tile, npts - i0);
        const int64_t ldt = round32(nt);
        const double* c = coords + 3 * i0;
        const double* w = weights + i0;
        wb::AoArgs ao;
        ao.coords = c; ao.npts = nt; ao.ld = ldt; ao.nbas = h->nbas;
        ao.sh_l = h->sh_l; ao.sh_np = h->sh_np; ao.sh_nc = h->sh_nc;
        ao.sh_eoff = h->sh_eoff; ao.sh_coff = h->sh_coff; ao.sh_ao0 = h->sh_ao0;
        ao.sh_ctr = h->sh_ctr; ao.exps = h->exps; ao.coeffs = h->coeffs; ao.X = X;
        ao.nao = nao;
        if ((st = phase_to(0)) != WB_OK) return st;
        WB_CUDA(wb::launch_ao_eval(ao, s));
        launches += 1;
        if ((st = phase_to(1)) != WB_OK) return st;
        if (oz_f) {
            const int r = wb::ozaki_f_gemm(
                h->cublas, X, qd, nao, ldt, F32, at<void>(workspace, L.oz), s,
                at<unsigned long long>(workspace, L.counters) + 3 * wb::NCLASS);
            if (r) return fail(r >= 1000 ? WB_ERR_CUBLAS : WB_ERR_CUDA,
                               "ozaki F GEMM failed, code " + std::to_string(r));
            launches += wb::ozaki_f_launches();
        } else {
            // F(g, mu) = sum_l X(g, l) QD(l, mu); QD row-major = col-major QD^T
            WB_CUBLAS(cublasDgemm(h->cublas, CUBLAS_OP_N, CUBLAS_OP_T, (int)ldt,
                                  nao, nao, &one, X, (int)ldt, qd, nao, &zero,
                                  F64, (int)ldt));
            if ((st = phase_to(2)) != WB_OK) return st;
            WB_CUDA(wb::launch_f64_to_f32(F64, F32, (int64_t)nao * ldt, s));
            launches += 2;
        }
        if ((st = phase_to(3)) != WB_OK) return st;
        if ((st = tile_prep(h, c, w, nt, ldt, F32, workspace, L, s, &launches)) != WB_OK)
            return st;
        // K += X^T (w o G) of omega j from the G in Gsrc; the X slices of
        // this tile serve every omega after the first
        bool x_sliced = false;
        auto k_gemm = [&](int j, const float* Gsrc) -> int {
            double* Kj = k_out + kk * j;
            int rs;
            if (oz_k) {
                if ((rs = phase_to(5)) != WB_OK) return rs;
                const int r = wb::ozaki_k_gemm(h->cublas, X, Gsrc, w, nao, ldt, nt,
                                               i0 == 0 ? 0 : 1, Kj,
                                               at<void>(workspace, L.oz), s, x_sliced);
                if (r) return fail(r >= 1000 ? WB_ERR_CUBLAS : WB_ERR_CUDA,
                                   "ozaki K GEMM failed, code " + std::to_string(r));
                x_sliced = true;
                launches += 2 + wb::kOzSlices;
            } else {
                if ((rs = phase_to(4)) != WB_OK) return rs;
                WB_CUDA(wb::launch_weight_g(Gsrc, w, nt, ldt, nao, F64, s));
                if ((rs = phase_to(5)) != WB_OK) return rs;
                // K(mu, nu) += sum_g X(g, mu) WG(g, nu); written row-major
                const double* beta = i0 == 0 ? &zero : &one;
                WB_CUBLAS(cublasDgemm(h->cublas, CUBLAS_OP_T, CUBLAS_OP_N, nao, nao,
                                      (int)ldt, &one, F64, (int)ldt, X, (int)ldt,
                                      beta, Kj, nao));
                launches += 2;
            }
            return phase_to(3);
        };
        for (int j = 0; j < nomega;) {
            if (h->dual_ok && j + 1 < nomega) {
                // two omegas in one pass of the class kernels; slot a (the
                // all-far-first branch order) takes the smaller omega
                int ja = j, jb = j + 1;
                if (omegas[jb] < omegas[ja]) std::swap(ja, jb);
                if ((st = prepare_omega_dual(h, omegas[ja], omegas[jb], workspace, L,
                                             s)) != WB_OK)
                    return st;
                launches += 3;
                if ((st = run_g_classes_dual(h, nt, ldt, F32, G32, G32b, omegas[ja],
                                             omegas[jb], tile_tol, workspace, L, s,
                                             &launches)) != WB_OK)
                    return st;
                ntasks += 2 * (ldt / 32) * (int64_t)h->hp.npairs;
                if (oz_k) {
                    // both omegas' w o G against the same X in one split
                    if ((st = phase_to(5)) != WB_OK) return st;
                    const float* Gs[2] = {G32, G32b};
                    double* Ks[2] = {k_out + kk * ja, k_out + kk * jb};
                    const int r = wb::ozaki_k_gemm_multi(
                        h->cublas, X, Gs, 2, w, nao, ldt, nt, i0 == 0 ? 0 : 1, Ks,
                        at<void>(workspace, L.oz), s, x_sliced);
                    if (r) return fail(r >= 1000 ? WB_ERR_CUBLAS : WB_ERR_CUDA,
                                       "ozaki K GEMM failed, code " + std::to_string(r));
                    x_sliced = true;
                    launches += 3 + wb::kOzSlices;
                    if ((st = phase_to(3)) != WB_OK) return st;
                } else {
                    if ((st = k_gemm(ja, G32)) != WB_OK) return st;
                    if ((st = k_gemm(jb, G32b)) != WB_OK) return st;
                }
                j += 2;
                continue;
            }
            if ((st = prepare_omega(h, omegas[j], workspace, L, s)) != WB_OK) return st;
            launches += 2;
            if ((st = run_g_classes(h, nt, ldt, F32, G32, omegas[j], tile_tol,
                                    workspace, L, s, &launches)) != WB_OK)
                return st;
            ntasks += (ldt / 32) * (int64_t)h->hp.npairs;
            if ((st = k_gemm(j, G32)) != WB_OK) return st;
            j += 1;
        }
    }
    if ((st = mark()) != WB_OK) return st;
    if (prof)
        for (int i = 0; i < 2; ++i) cudaEventDestroy(ev[i]);
    st = read_stats(h, workspace, L, ntasks, s, stats, launches);
    if (st == WB_OK && prof)
        for (int i = 0; i < 6; ++i) stats->phase_ms[i] = phase[i];
    return st;
}

int wb_cosx_set_class_variant(wb_cosx* h, int cls, int dual, int staged) {
    if (!h || cls < 0 || cls >= wb::NCLASS || dual < 0 || dual > 1 || staged < 0 ||
        staged > 1)
        return fail(WB_ERR_INVALID_ARGUMENT, "wb_cosx_set_class_variant: bad arguments");
    const int c = cls;
    if (dual && !(h->stage_smem2[c] > 0 && h->blocks_per_sm2[c] >= 1))
        return fail(WB_ERR_UNSUPPORTED, "wb_cosx_set_class_variant: class " +
                                            std::to_string(c) +
                                            " has no two-omega kernel for this molecule");
    size_t smem = 0;
    if (staged) {
        smem = (size_t)(128 / 32) * 2 * h->recmax[c] * sizeof(float4);
        if (h->recmax[c] <= 0 || smem > kStageMaxBytes)
            return fail(WB_ERR_UNSUPPORTED, "wb_cosx_set_class_variant: class " +
                                                std::to_string(c) +
                                                " records do not fit the staged kernel");
    }
    int n[2];
    for (int f = 0; f < 2; ++f) n[f] = wb::cosx_class_blocks_per_sm(c, f == 1, smem);
    if (n[0] == 0 || n[1] == 0)
        return fail(WB_ERR_UNSUPPORTED, "wb_cosx_set_class_variant: no occupancy");
    h->stage_smem[c] = smem;
    for (int f = 0; f < 2; ++f) h->blocks_per_sm[c][f] = n[f];
    h->dual_cls[c] = dual != 0;
    return WB_OK;
}

int wb_cosx_get_class_variant(const wb_cosx* h, int cls, int* dual, int* staged) {
    if (!h || cls < 0 || cls >= wb::NCLASS || !dual || !staged)
        return fail(WB_ERR_INVALID_ARGUMENT, "wb_cosx_get_class_variant: bad arguments");
    *dual = h->dual_cls[cls] ? 1 : 0;
    *staged = h->stage_smem[cls] > 0 ? 1 : 0;
    return WB_OK;
}

size_t wb_cosx_fp64_workspace_bytes(const wb_cosx* h, int64_t npts) {
    if (!h || npts < 0) return 0;
    return ws_layout_fp64(h, round32(std::max<int64_t>(npts, 1))).total;
}

int wb_cosx_get_k_fp64(wb_cosx* h, const double* coords, const double* weights,
                       int64_t npts, const double* qd, int nomega,
                       const double* omegas, double tile_tol, double* k_out,
                       void* workspace, size_t workspace_bytes, void* stream,
                       wb_cosx_stats* stats) {
    if (!h || !k_out || !qd || npts < 0 || (npts && (!coords || !weights)) ||
        nomega < 1 || !omegas)
        return fail(WB_ERR_INVALID_ARGUMENT, "wb_cosx_get_k_fp64: bad arguments");
    for (int j = 0; j < nomega; ++j)
        if (!(omegas[j] >= 0.0))
            return fail(WB_ERR_INVALID_ARGUMENT, "wb_cosx_get_k_fp64: omega must be >= 0");
    if (!(tile_tol >= 0.0))
        return fail(WB_ERR_INVALID_ARGUMENT, "wb_cosx_get_k_fp64: tile_tol must be >= 0");
    const int64_t ld = round32(std::max<int64_t>(npts, 1));
    if (ld > INT32_MAX - 64)
        return fail(WB_ERR_UNSUPPORTED, "wb_cosx_get_k_fp64: above 2^31 points");
    const WsLayout64 L = ws_layout_fp64(h, ld);
    if (!workspace || workspace_bytes < L.total)
        return fail(WB_ERR_WORKSPACE, "wb_cosx_get_k_fp64: workspace needs " +
                                          std::to_string(L.total) + " bytes");
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const int nao = h->hp.nao;
    const size_t kk = (size_t)nao * nao;
    WB_CUDA(cudaMemsetAsync(at<void>(workspace, L.base.counters), 0,
                            sizeof(unsigned long long) * kCounterWords, s));
    int launches = 1;
    if (npts == 0) {
        WB_CUDA(cudaMemsetAsync(k_out, 0, sizeof(double) * kk * nomega, s));
        return read_stats(h, workspace, L.base, 0, s, stats, launches);
    }
    int st = ensure_fp64(h);
    if (st != WB_OK) return st;
    WB_CUBLAS(cublasSetStream(h->cublas, s));
    WB_CUBLAS(cublasSetMathMode(h->cublas, CUBLAS_DEFAULT_MATH));
    double* X = at<double>(workspace, L.X);
    double* F64 = at<double>(workspace, L.F64);
    float* F32 = at<float>(workspace, L.F32);
    double* G64 = at<double>(workspace, L.G64);
    double* WG = at<double>(workspace, L.WG);
    const double one = 1.0, zero = 0.0;
    wb::AoArgs ao;
    ao.coords = coords; ao.npts = npts; ao.ld = ld; ao.nbas = h->nbas;
    ao.sh_l = h->sh_l; ao.sh_np = h->sh_np; ao.sh_nc = h->sh_nc;
    ao.sh_eoff = h->sh_eoff; ao.sh_coff = h->sh_coff; ao.sh_ao0 = h->sh_ao0;
    ao.sh_ctr = h->sh_ctr; ao.exps = h->exps; ao.coeffs = h->coeffs; ao.X = X;
    ao.nao = nao;
    WB_CUDA(wb::launch_ao_eval(ao, s));
    // F = X QD in FP64 (no rounding); its FP32 copy feeds only the block
    // statistics of the screen, as in the mixed-precision path
    WB_CUBLAS(cublasDgemm(h->cublas, CUBLAS_OP_N, CUBLAS_OP_T, (int)ld, nao, nao,
                          &one, X, (int)ld, qd, nao, &zero, F64, (int)ld));
    WB_CUDA(wb::launch_f64_to_f32(F64, F32, (int64_t)nao * ld, s));
    wb::BlockStatsOut bo;
    for (int b = 0; b < 3; ++b) {
        bo.cr[b] = at<float4>(workspace, L.base.subcr[b]);
        bo.msh[b] = at<float>(workspace, L.base.msh[b]);
    }
    WB_CUDA(wb::launch_sub_stats(coords, weights, F32, npts, ld, h->hp.nvshell,
                                 h->vs_ao0, h->vs_nf, bo, s));
    launches += 4;
    wb::CosxF64Args a;
    std::memset(&a, 0, sizeof(a));
    a.F = F64;
    a.G = G64;
    a.coords = coords;
    a.ld = ld;
    a.npts = (int)npts;
    a.khdr = h->khdr;
    a.pshell = h->pshell;
    a.ptau = h->ptau;
    a.bnd = h->bnd;
    a.bpref = h->bpref;
    a.blk_cr = bo.cr[0];
    a.blk_msh = bo.msh[0];
    a.nblk = (int)(ld / 32);
    a.nvshell = h->hp.nvshell;
    a.tol = tile_tol > 0.0 ? (float)(tile_tol / 1.001) : 0.0f;
    if (tile_tol > 0.0 && a.tol <= 0.0f) a.tol = 1e-38f;
    for (int c = 0; c < wb::NCLASS; ++c) {
        a.pp_begin[c] = h->hp.cls[c].pp_begin;
        a.e_base[c] = h->f64_ebase[c];
    }
    a.P = h->f64_P;
    a.p = h->p;
    a.pref = h->pref;
    a.E = h->f64_E;
    a.boys = h->f64_boys;
    a.c2s = h->f64_boys + (size_t)wb::kBoys64Nodes * wb::kBoys64Cols;
    a.pflops = h->pflops;
    a.pnint = h->pnint;
    a.counters = at<unsigned long long>(workspace, L.base.counters);
    a.work = at<int>(workspace, L.base.work);
    int64_t ntasks = 0;
    for (int j = 0; j < nomega; ++j) {
        a.omega = omegas[j];
        WB_CUDA(cudaMemsetAsync(G64, 0, sizeof(double) * (size_t)nao * ld, s));
        WB_CUDA(cudaMemsetAsync(a.work, 0, sizeof(int) * wb::NCLASS, s));
        launches += 2;
        for (int c = 0; c < wb::NCLASS; ++c) {
            const int pb = h->hp.cls[c].pair_begin, pe = h->hp.cls[c].pair_end;
            if (pe <= pb) continue;
            WB_CUDA(wb::launch_cosx_fp64_class(c, a, pb, pe, h->nsm, s));
            ++launches;
        }
        ntasks += (ld / 32) * (int64_t)h->hp.npairs;
        WB_CUDA(wb::launch_weight_g64(G64, weights, npts, ld, nao, WG, s));
        WB_CUBLAS(cublasDgemm(h->cublas, CUBLAS_OP_T, CUBLAS_OP_N, nao, nao, (int)ld,
                              &one, WG, (int)ld, X, (int)ld, &zero, k_out + kk * j,
                              nao));
        launches += 2;
    }
    return read_stats(h, workspace, L.base, ntasks, s, stats, launches);
}

size_t wb_cosx_batch_workspace_bytes(const wb_cosx* h, int64_t npts,
                                     size_t* scratch_bytes) {
    if (!h || npts < 1) return 0;
    const WsLayout L = ws_layout(h, round32(npts), true);
    if (scratch_bytes) *scratch_bytes = L.total - L.oz;
    return L.oz;
}

int wb_cosx_batch_create(int nmol, wb_cosx* const* handles,
                         const double* const* coords, const double* const* weights,
                         const int64_t* npts, void* const* workspaces,
                         const size_t* workspace_bytes, void* scratch,
                         size_t scratch_bytes, int nomega, const double* omegas,
                         double tile_tol, int flags, void* stream,
                         wb_cosx_batch** out) {
    if (!out || nmol < 1 || !handles || !coords || !weights || !npts || !workspaces ||
        !workspace_bytes || !scratch || !omegas || nomega < 1 || nomega > 2 ||
        !(tile_tol >= 0.0))
        return fail(WB_ERR_INVALID_ARGUMENT, "wb_cosx_batch_create: bad arguments");
    *out = nullptr;
    for (int j = 0; j < nomega; ++j)
        if (!(omegas[j] >= 0.0))
            return fail(WB_ERR_INVALID_ARGUMENT,
                        "wb_cosx_batch_create: omega must be >= 0");
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    wb_cosx_batch* b = new wb_cosx_batch();
    b->nmol = nmol;
    b->nom = nomega;
    b->om[0] = omegas[0];
    if (nomega == 2) {
        b->om[1] = omegas[1];
        if (omegas[1] < omegas[0]) {
            std::swap(b->om[0], b->om[1]);
            b->kidx[0] = 1;
            b->kidx[1] = 0;
        }
    }
    b->tol = tile_tol;
    b->gemm = flags & 3;
    b->scratch = scratch;
    for (int m = 0; m < nmol; ++m) {
        wb_cosx* h = handles[m];
        if (!h || !coords[m] || !weights[m] || npts[m] < 1 || !workspaces[m])
            return batch_fail(b, fail(WB_ERR_INVALID_ARGUMENT,
                                      "wb_cosx_batch_create: molecule " +
                                          std::to_string(m) + ": bad arguments"));
        if (h->device != handles[0]->device)
            return batch_fail(b, fail(WB_ERR_INVALID_ARGUMENT,
                                      "wb_cosx_batch_create: handles on different devices"));
        for (int k = 0; k < m; ++k)
            if (handles[k] == h)
                return batch_fail(b, fail(WB_ERR_INVALID_ARGUMENT,
                                          "wb_cosx_batch_create: a handle appears twice"));
        const int64_t ld = round32(npts[m]);
        if (ld > INT32_MAX - 64)
            return batch_fail(b, fail(WB_ERR_UNSUPPORTED,
                                      "wb_cosx_batch_create: above 2^31 points"));
        const WsLayout L = ws_layout(h, ld, true);
        if (workspace_bytes[m] < L.oz || scratch_bytes < L.total - L.oz)
            return batch_fail(b, fail(WB_ERR_WORKSPACE,
                                      "wb_cosx_batch_create: molecule " +
                                          std::to_string(m) + " needs " +
                                          std::to_string(L.oz) + " workspace and " +
                                          std::to_string(L.total - L.oz) +
                                          " scratch bytes"));
        b->h.push_back(h);
        b->coords.push_back(coords[m]);
        b->weights.push_back(weights[m]);
        b->npts.push_back(npts[m]);
        b->ld.push_back(ld);
        b->ws.push_back(workspaces[m]);
        b->L.push_back(L);
    }
    // per class: the kernel variant every molecule runs, the largest task
    // record, the blocks (items) over the molecules
    double work[wb::NCLASS] = {0};
    for (int c = 0; c < wb::NCLASS; ++c) {
        bool dual = nomega == 2, staged = true;
        for (int m = 0; m < nmol; ++m) {
            const wb_cosx* h = b->h[m];
            if (h->hp.cls[c].pair_end <= h->hp.cls[c].pair_begin) continue;
            b->has[c] = true;
            dual = dual && h->dual_ok && h->dual_cls[c];
            staged = staged && h->stage_smem[c] > 0;
            b->rmax[c] = std::max(b->rmax[c], h->recmax[c]);
            b->rmax2[c] = std::max(b->rmax2[c], h->recmax2[c]);
            for (int k = h->hp.cls[c].pair_begin; k < h->hp.cls[c].pair_end; ++k)
                work[c] += (double)h->hp.pflops[k] * (double)b->npts[m];
        }
        const size_t sm = (size_t)(128 / 32) * 2 * b->rmax[c] * sizeof(float4);
        const size_t sm2 = (size_t)(128 / 32) * 2 * b->rmax2[c] * sizeof(float4);
        b->dual[c] = b->has[c] && dual && sm2 <= kStageMaxBytes;
        b->smem2[c] = b->dual[c] ? sm2 : 0;
        b->smem[c] = (b->has[c] && staged && sm <= kStageMaxBytes) ? sm : 0;
        b->order[c] = c;
    }
    std::stable_sort(b->order, b->order + wb::NCLASS,
                     [&](int x, int y) { return work[x] > work[y]; });
    // host argument blocks (slot a, slot b) and item offsets
    std::vector<wb::CosxArgs> args(2 * (size_t)nmol);
    std::vector<int> off((size_t)wb::NCLASS * (nmol + 1), 0);
    for (int m = 0; m < nmol; ++m) {
        wb_cosx* h = b->h[m];
        const WsLayout& L = b->L[m];
        wb::CosxArgs a = make_args(h, b->ws[m], L, b->ld[m], b->npts[m],
                                   at<float>(b->ws[m], L.F32), tile_tol);
        wb::CosxArgs bb = a;
        for (int c = 0; c < wb::NCLASS; ++c) {
            bb.rec[c] = at<float4>(b->ws[m], L.recb) + h->hp.rec_off[c];
            bb.Gcls[c] = a.Gcls2[c];
#if WB_COSX_SPLIT
            bb.GclsH[c] = a.Gcls2H[c];
#endif
        }
        args[m] = a;
        args[nmol + m] = bb;
    }
    for (int c = 0; c < wb::NCLASS; ++c) {
        int* o = off.data() + (size_t)c * (nmol + 1);
        for (int m = 0; m < nmol; ++m) {
            const wb_cosx* h = b->h[m];
            int n = 0;
            if (h->hp.cls[c].pair_end > h->hp.cls[c].pair_begin) {
                const int pc = b->dual[c] ? h->pts2[c] : h->pts[c];
                n = (WB_COSX_SPLIT ? 2 : 1) * args[m].nblk[pc == 4 ? 2 : pc - 1];
            }
            if ((int64_t)o[m] + n > INT32_MAX)
                return batch_fail(b, fail(WB_ERR_UNSUPPORTED,
                                          "wb_cosx_batch_create: too many blocks"));
            o[m + 1] = o[m] + n;
        }
        b->items[c] = o[nmol];
    }
    int64_t stride = 1;
    for (int c = 0; c < wb::NCLASS; ++c) stride = std::max<int64_t>(stride, b->items[c]);
    b->stride = stride;
    const size_t args_b = align256(sizeof(wb::CosxArgs) * args.size());
    const size_t off_b = align256(sizeof(int) * off.size());
    const size_t work_b = align256(sizeof(int) * 2 * wb::NCLASS);
    const size_t cost_b = align256(sizeof(float) * wb::NCLASS * stride);
    const size_t order_b = align256(sizeof(int) * wb::NCLASS * stride);
    cudaError_t e = cudaMalloc(&b->block, args_b + off_b + work_b + cost_b + order_b);
    if (e != cudaSuccess) return batch_fail(b, cuda_fail(e, "wb_cosx_batch_create"));
    char* blk = static_cast<char*>(b->block);
    b->d_args = reinterpret_cast<wb::CosxArgs*>(blk);
    b->d_off = reinterpret_cast<int*>(blk + args_b);
    b->d_work = reinterpret_cast<int*>(blk + args_b + off_b);
    b->d_cost = reinterpret_cast<float*>(blk + args_b + off_b + work_b);
    b->d_order = reinterpret_cast<int*>(blk + args_b + off_b + work_b + cost_b);
    // every block records its kept model flops at its item index, the
    // order of the next run
    for (int m = 0; m < nmol; ++m)
        for (int c = 0; c < wb::NCLASS; ++c) {
            float* row = b->d_cost + (size_t)c * stride + off[(size_t)c * (nmol + 1) + m];
            args[m].bcost[c] = row;
            args[nmol + m].bcost[c] = row;
        }
    e = cudaMemcpy(b->d_args, args.data(), sizeof(wb::CosxArgs) * args.size(),
                   cudaMemcpyHostToDevice);
    if (e == cudaSuccess)
        e = cudaMemcpy(b->d_off, off.data(), sizeof(int) * off.size(),
                       cudaMemcpyHostToDevice);
    if (e != cudaSuccess) return batch_fail(b, cuda_fail(e, "wb_cosx_batch_create"));
    // what stays fixed for the plan's life: AO values, grid coordinates
    // (hi / lo), the omega records of both slots
    for (int m = 0; m < nmol; ++m) {
        wb_cosx* h = b->h[m];
        const WsLayout& L = b->L[m];
        void* ws = b->ws[m];
        wb::AoArgs ao;
        ao.coords = b->coords[m]; ao.npts = b->npts[m]; ao.ld = b->ld[m];
        ao.nbas = h->nbas; ao.sh_l = h->sh_l; ao.sh_np = h->sh_np;
        ao.sh_nc = h->sh_nc; ao.sh_eoff = h->sh_eoff; ao.sh_coff = h->sh_coff;
        ao.sh_ao0 = h->sh_ao0; ao.sh_ctr = h->sh_ctr; ao.exps = h->exps;
        ao.coeffs = h->coeffs; ao.X = at<double>(ws, L.X); ao.nao = h->hp.nao;
        e = wb::launch_ao_eval(ao, s);
        if (e == cudaSuccess)
            e = wb::launch_grid_prep(b->coords[m], b->npts[m], b->ld[m],
                                     at<float>(ws, L.gh), at<float>(ws, L.gl), s);
        if (e != cudaSuccess) return batch_fail(b, cuda_fail(e, "wb_cosx_batch_create"));
        wb::RecPack P;
        for (int c = 0; c < wb::NCLASS; ++c) {
            P.pp_begin[c] = h->hp.cls[c].pp_begin;
            P.pp_end[c] = h->hp.cls[c].pp_end;
            P.stride[c] = wb::kRecStride[c];
            P.nom[c] = wb::kRecNom[c];
            P.ne[c] = wb::kRecNe[c];
            P.rec_off[c] = h->hp.rec_off[c];
            P.e_off[c] = h->hp.cls[c].e_base / 4;
        }
        const size_t slot_rec[2] = {L.rec, L.recb};
        const size_t slot_om[2] = {L.om, L.om2};
        for (int w = 0; w < nomega && e == cudaSuccess; ++w) {
            e = wb::launch_omega(h->hp.npp, h->p, h->pref, b->om[w],
                                 at<float4>(ws, slot_om[w]), s);
            if (e == cudaSuccess)
                e = wb::launch_pack_records(P, h->hp.npp, h->geo,
                                            at<float4>(ws, slot_om[w]), h->E,
                                            at<float4>(ws, slot_rec[w]), s);
        }
        if (e == cudaSuccess && nomega == 2) {
            for (int c = 0; c < wb::NCLASS; ++c) {
                P.stride[c] = wb::kRecStride2[c];
                P.rec_off[c] = h->hp.rec_off2[c];
            }
            e = wb::launch_pack_records2(P, h->hp.npp, h->geo, at<float4>(ws, L.om),
                                         at<float4>(ws, L.om2), h->E,
                                         at<float4>(ws, L.rec2), s);
        }
        if (e != cudaSuccess) return batch_fail(b, cuda_fail(e, "wb_cosx_batch_create"));
    }
    e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return batch_fail(b, cuda_fail(e, "wb_cosx_batch_create"));
    *out = b;
    return WB_OK;
}

int wb_cosx_batch_run(wb_cosx_batch* b, const double* const* qd,
                      double* const* k_out, void* stream, wb_cosx_stats* stats) {
    if (!b || !qd || !k_out)
        return fail(WB_ERR_INVALID_ARGUMENT, "wb_cosx_batch_run: bad arguments");
    int active = 0;
    for (int m = 0; m < b->nmol; ++m) {
        if (qd[m] && !k_out[m])
            return fail(WB_ERR_INVALID_ARGUMENT, "wb_cosx_batch_run: null output");
        active += qd[m] ? 1 : 0;
    }
    if (!active)
        return fail(WB_ERR_INVALID_ARGUMENT, "wb_cosx_batch_run: no molecule to build");
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const int nmol = b->nmol;
    int launches = 0;
    const double one = 1.0, zero = 0.0;
    // per molecule: F = fl32(X QD) and the block statistics
    for (int m = 0; m < nmol; ++m) {
        wb_cosx* h = b->h[m];
        const WsLayout& L = b->L[m];
        void* ws = b->ws[m];
        const int nao = h->hp.nao;
        const int64_t ld = b->ld[m];
        WB_CUBLAS(cublasSetStream(h->cublas, s));
        WB_CUBLAS(cublasSetMathMode(h->cublas, CUBLAS_DEFAULT_MATH));
        if (stats)
            WB_CUDA(cudaMemsetAsync(at<void>(ws, L.counters), 0,
                                    sizeof(unsigned long long) * kCounterWords, s));
        const double* X = at<double>(ws, L.X);
        float* F32 = at<float>(ws, L.F32);
        if (!qd[m]) {
            // an inactive molecule: F = 0, so its screen keeps no task
            WB_CUDA(cudaMemsetAsync(F32, 0, sizeof(float) * (size_t)nao * ld, s));
        } else if (b->gemm == WB_K_GEMM_OZAKI_BF16 && wb::ozaki_f_supported(nao)) {
            const int r = wb::ozaki_f_gemm(
                h->cublas, X, qd[m], nao, ld, F32, b->scratch, s,
                at<unsigned long long>(ws, L.counters) + 3 * wb::NCLASS);
            if (r) return fail(r >= 1000 ? WB_ERR_CUBLAS : WB_ERR_CUDA,
                               "ozaki F GEMM failed, code " + std::to_string(r));
            launches += wb::ozaki_f_launches();
        } else {
            double* F64 = static_cast<double*>(b->scratch);
            WB_CUBLAS(cublasDgemm(h->cublas, CUBLAS_OP_N, CUBLAS_OP_T, (int)ld, nao, nao,
                                  &one, X, (int)ld, qd[m], nao, &zero, F64, (int)ld));
            WB_CUDA(wb::launch_f64_to_f32(F64, F32, (int64_t)nao * ld, s));
            launches += 2;
        }
        wb::BlockStatsOut bo;
        for (int k = 0; k < 3; ++k) {
            bo.cr[k] = at<float4>(ws, L.subcr[k]);
            bo.msh[k] = at<float>(ws, L.msh[k]);
        }
        WB_CUDA(wb::launch_sub_stats(b->coords[m], b->weights[m], F32, b->npts[m], ld,
                                     h->hp.nvshell, h->vs_ao0, h->vs_nf, bo, s));
        launches += 1;
    }
    // every class: one launch over all molecules (two for the classes
    // without a two-omega kernel)
    WB_CUDA(cudaMemsetAsync(b->d_work, 0, sizeof(int) * 2 * wb::NCLASS, s));
    launches += 1;
    const wb_cosx* h0 = b->h[0];
    for (int i = 0; i < wb::NCLASS; ++i) {
        const int c = b->order[i];
        if (!b->has[c] || b->items[c] == 0) continue;
        const int want = (b->items[c] + 3) / 4;
        const int* off = b->d_off + (size_t)c * (nmol + 1);
        const int* order = b->ordered ? b->d_order + (size_t)c * b->stride : nullptr;
        if (b->dual[c]) {
            const int cap = std::max(1, h0->blocks_per_sm2[c]) * h0->nsm;
            WB_CUDA(wb::launch_cosx_class_batch(c, b->d_args, off, nmol,
                                                b->d_work + 2 * c, b->rmax2[c], order,
                                                std::max(1, std::min(want, cap)), s,
                                                false, b->smem2[c], true));
            launches += 1;
        } else {
            for (int w = 0; w < b->nom; ++w) {
                const bool far = b->om[w] == 0.0;
                const int cap = std::max(1, h0->blocks_per_sm[c][far ? 1 : 0]) * h0->nsm;
                WB_CUDA(wb::launch_cosx_class_batch(
                    c, b->d_args + (size_t)w * nmol, off, nmol, b->d_work + 2 * c + w,
                    b->rmax[c], order, std::max(1, std::min(want, cap)), s, far,
                    b->smem[c], false));
                launches += 1;
            }
        }
    }
    {   // the next run takes each class's items costliest first
        wb::BlockOrderArgs P;
        P.cost = b->d_cost;
        P.order = b->d_order;
        P.stride = b->stride;
        for (int c = 0; c < wb::NCLASS; ++c) P.n[c] = b->has[c] ? b->items[c] : 0;
        WB_CUDA(wb::launch_block_order(P, s));
        launches += 1;
        b->ordered = true;
    }
    // per molecule: G of each slot, then K
    for (int m = 0; m < nmol; ++m) {
        if (!qd[m]) continue;
        wb_cosx* h = b->h[m];
        const WsLayout& L = b->L[m];
        void* ws = b->ws[m];
        const int nao = h->hp.nao;
        const int64_t ld = b->ld[m];
        const size_t kk = (size_t)nao * nao;
        const double* X = at<double>(ws, L.X);
        float* Gs[2] = {at<float>(ws, L.G32), at<float>(ws, L.G32b)};
        const size_t gcl[2] = {L.gcls, L.gcls2};
        double* Ks[2] = {k_out[m] + kk * b->kidx[0], k_out[m] + kk * b->kidx[1]};
#if WB_COSX_SPLIT
        const size_t gclH[2] = {L.gclsH, L.gcls2H};
        for (int w = 0; w < b->nom; ++w)
            WB_CUDA(wb::launch_gsum2(at<float>(ws, gcl[w]), at<float>(ws, gclH[w]),
                                     h->gsrc, nao, ld, Gs[w], s));
#else
        for (int w = 0; w < b->nom; ++w)
            WB_CUDA(wb::launch_gsum(at<float>(ws, gcl[w]), h->gsrc, nao, ld, Gs[w], s));
#endif
        launches += b->nom;
        if (b->gemm == WB_K_GEMM_OZAKI_BF16) {
            const float* Gc[2] = {Gs[0], Gs[1]};
            const int r = wb::ozaki_k_gemm_multi(h->cublas, X, Gc, b->nom, b->weights[m],
                                                 nao, ld, b->npts[m], 0, Ks,
                                                 b->scratch, s, false);
            if (r) return fail(r >= 1000 ? WB_ERR_CUBLAS : WB_ERR_CUDA,
                               "ozaki K GEMM failed, code " + std::to_string(r));
            launches += 3 + wb::kOzSlices;
        } else {
            double* WG = static_cast<double*>(b->scratch);
            for (int w = 0; w < b->nom; ++w) {
                WB_CUDA(wb::launch_weight_g(Gs[w], b->weights[m], b->npts[m], ld, nao,
                                            WG, s));
                WB_CUBLAS(cublasDgemm(h->cublas, CUBLAS_OP_T, CUBLAS_OP_N, nao, nao,
                                      (int)ld, &one, WG, (int)ld, X, (int)ld, &zero,
                                      Ks[w], nao));
                launches += 2;
            }
        }
    }
    if (!stats) return WB_OK;
    std::memset(stats, 0, sizeof(*stats));
    for (int m = 0; m < nmol; ++m) {
        wb_cosx_stats st;
        const int r = read_stats(b->h[m], b->ws[m], b->L[m],
                                 b->nom * (b->ld[m] / 32) * (int64_t)b->h[m]->hp.npairs,
                                 s, &st, 0);
        if (r != WB_OK) return r;
        stats->tasks_total += st.tasks_total;
        stats->tasks_kept += st.tasks_kept;
        stats->integrals += st.integrals;
        stats->model_flops += st.model_flops;
        for (int c = 0; c < wb::NCLASS; ++c) {
            stats->tasks_kept_class[c] += st.tasks_kept_class[c];
            stats->model_flops_class[c] += st.model_flops_class[c];
        }
    }
    stats->kernel_launches = launches;
    return WB_OK;
}

int wb_cosx_batch_destroy(wb_cosx_batch* b) {
    if (!b) return WB_OK;
    if (b->block) cudaFree(b->block);
    delete b;
    return WB_OK;
}

size_t wb_cosx_k_grad_workspace_bytes(const wb_cosx* h, int64_t npts, int natm) {
    if (!h || npts < 0 || natm < 1) return 0;
    const int64_t ld = round32(std::max<int64_t>(npts, 1));
    const WsLayout64 L = ws_layout_fp64(h, ld);
    const size_t n = (size_t)h->hp.nao * ld;
    return align256(L.total + sizeof(double) * 4 * n) +
           align256(sizeof(double) * (size_t)(ld / 32) * natm * 3) +
           align256(sizeof(double) * 3 * (size_t)h->hp.nao);
}

int wb_cosx_k_grad(wb_cosx* h, const double* coords, const double* weights,
                   int64_t npts, const double* dm, double omega, double tile_tol,
                   int natm, double* grad_out, void* workspace,
                   size_t workspace_bytes, void* stream) {
    if (!h || !dm || !grad_out || npts < 1 || !coords || !weights || natm < 1 ||
        !(omega >= 0.0) || !(tile_tol >= 0.0))
        return fail(WB_ERR_INVALID_ARGUMENT, "wb_cosx_k_grad: bad arguments");
    for (const wb::VShell& v : h->hp.vsh)
        if (v.atom >= natm)
            return fail(WB_ERR_INVALID_ARGUMENT, "wb_cosx_k_grad: natm below the basis atoms");
    const int64_t ld = round32(npts);
    if (ld > INT32_MAX - 64)
        return fail(WB_ERR_UNSUPPORTED, "wb_cosx_k_grad: above 2^31 points");
    const size_t need = wb_cosx_k_grad_workspace_bytes(h, npts, natm);
    if (!workspace || workspace_bytes < need)
        return fail(WB_ERR_WORKSPACE, "wb_cosx_k_grad: workspace needs " +
                                          std::to_string(need) + " bytes");
    int st = ensure_fp64(h);
    if (st != WB_OK) return st;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const int nao = h->hp.nao;
    const size_t n = (size_t)nao * ld;
    // the FP64 form's layout, then the AO values and their x, y, z
    // gradients (4, nao, ld), the per-block gradient rows and the AO sums
    const WsLayout64 L = ws_layout_fp64(h, ld);
    char* base = static_cast<char*>(workspace);
    double* Xd = reinterpret_cast<double*>(base + L.total);     // (4, nao, ld)
    double* gbuf = reinterpret_cast<double*>(base + align256(L.total + sizeof(double) * 4 * n));
    const int nblk = (int)(ld / 32);
    double* aodot = reinterpret_cast<double*>(
        reinterpret_cast<char*>(gbuf) + align256(sizeof(double) * (size_t)nblk * natm * 3));
    double* F64 = at<double>(workspace, L.F64);
    float* F32 = at<float>(workspace, L.F32);
    double* G64 = at<double>(workspace, L.G64);
    double* H = at<double>(workspace, L.WG);
    WB_CUBLAS(cublasSetStream(h->cublas, s));
    WB_CUBLAS(cublasSetMathMode(h->cublas, CUBLAS_DEFAULT_MATH));
    const double one = 1.0, zero = 0.0;
    wb::AoArgs ao;
    ao.coords = coords; ao.npts = npts; ao.ld = ld; ao.nbas = h->nbas;
    ao.sh_l = h->sh_l; ao.sh_np = h->sh_np; ao.sh_nc = h->sh_nc;
    ao.sh_eoff = h->sh_eoff; ao.sh_coff = h->sh_coff; ao.sh_ao0 = h->sh_ao0;
    ao.sh_ctr = h->sh_ctr; ao.exps = h->exps; ao.coeffs = h->coeffs; ao.X = Xd;
    ao.nao = nao;
    WB_CUDA(wb::launch_ao_eval_d1(ao, s));
    // F = X D (FP64); fl32(F) feeds the screen's block statistics only
    WB_CUBLAS(cublasDgemm(h->cublas, CUBLAS_OP_N, CUBLAS_OP_T, (int)ld, nao, nao, &one,
                          Xd, (int)ld, dm, nao, &zero, F64, (int)ld));
    WB_CUDA(wb::launch_f64_to_f32(F64, F32, (int64_t)n, s));
    wb::BlockStatsOut bo;
    for (int b = 0; b < 3; ++b) {
        bo.cr[b] = at<float4>(workspace, L.base.subcr[b]);
        bo.msh[b] = at<float>(workspace, L.base.msh[b]);
    }
    WB_CUDA(wb::launch_sub_stats(coords, weights, F32, npts, ld, h->hp.nvshell,
                                 h->vs_ao0, h->vs_nf, bo, s));
    const float tol = tile_tol > 0.0 ? std::max((float)(tile_tol / 1.001), 1e-38f) : 0.0f;
    int* work = at<int>(workspace, L.base.work);
    // G = A F by the FP64 class kernels
    wb::CosxF64Args a;
    std::memset(&a, 0, sizeof(a));
    a.F = F64; a.G = G64; a.coords = coords; a.ld = ld; a.npts = (int)npts;
    a.omega = omega; a.khdr = h->khdr; a.pshell = h->pshell; a.ptau = h->ptau;
    a.bnd = h->bnd; a.bpref = h->bpref; a.blk_cr = bo.cr[0]; a.blk_msh = bo.msh[0];
    a.nblk = nblk; a.nvshell = h->hp.nvshell; a.tol = tol;
    for (int c = 0; c < wb::NCLASS; ++c) {
        a.pp_begin[c] = h->hp.cls[c].pp_begin;
        a.e_base[c] = h->f64_ebase[c];
    }
    a.P = h->f64_P; a.p = h->p; a.pref = h->pref; a.E = h->f64_E; a.boys = h->f64_boys;
    a.c2s = h->f64_boys + (size_t)wb::kBoys64Nodes * wb::kBoys64Cols;
    a.pflops = h->pflops; a.pnint = h->pnint;
    a.counters = at<unsigned long long>(workspace, L.base.counters);
    a.work = work;
    WB_CUDA(cudaMemsetAsync(a.counters, 0, sizeof(unsigned long long) * kCounterWords, s));
    WB_CUDA(cudaMemsetAsync(G64, 0, sizeof(double) * n, s));
    WB_CUDA(cudaMemsetAsync(work, 0, sizeof(int) * wb::NCLASS, s));
    for (int c = 0; c < wb::NCLASS; ++c) {
        const int pb = h->hp.cls[c].pair_begin, pe = h->hp.cls[c].pair_end;
        if (pe > pb) WB_CUDA(wb::launch_cosx_fp64_class(c, a, pb, pe, h->nsm, s));
    }
    // X side: 1/2 sum_g w_g sum_{mu on C} grad X_g,mu (G D)_g,mu
    WB_CUBLAS(cublasDgemm(h->cublas, CUBLAS_OP_N, CUBLAS_OP_T, (int)ld, nao, nao, &one,
                          G64, (int)ld, dm, nao, &zero, H, (int)ld));
    WB_CUDA(cudaMemsetAsync(grad_out, 0, sizeof(double) * 3 * (size_t)natm, s));
    WB_CUDA(wb::launch_ao_dot(Xd, H, weights, npts, ld, nao, aodot, s));
    WB_CUDA(wb::launch_atom_sum(aodot, h->vs_ao0, h->vs_nf, h->vs_atom, h->hp.nvshell,
                                natm, 0.5, grad_out, s));
    // integral side
    wb::CosxGradArgs g;
    std::memset(&g, 0, sizeof(g));
    g.F = F64; g.coords = coords; g.weights = weights; g.ld = ld; g.npts = (int)npts;
    g.omega = omega; g.khdr = h->khdr; g.pshell = h->pshell; g.ptau = h->ptau;
    g.bnd = h->bnd; g.bpref = h->bpref; g.blk_cr = bo.cr[0]; g.blk_msh = bo.msh[0];
    g.nblk = nblk; g.nvshell = h->hp.nvshell; g.tol = tol;
    for (int c = 0; c < wb::NCLASS; ++c) g.pp_begin[c] = h->hp.cls[c].pp_begin;
    g.P = h->f64_P; g.p = h->p; g.pref = h->pref; g.alpha = h->f64_alpha;
    g.vs_xyz = h->f64_vsxyz; g.vs_atom = h->vs_atom; g.boys = h->f64_boys;
    g.c2s = a.c2s; g.gbuf = gbuf; g.natm = natm; g.work = work;
    WB_CUDA(cudaMemsetAsync(gbuf, 0, sizeof(double) * (size_t)nblk * natm * 3, s));
    WB_CUDA(cudaMemsetAsync(work, 0, sizeof(int) * wb::NCLASS, s));
    for (int c = 0; c < wb::NCLASS; ++c) {
        const int pb = h->hp.cls[c].pair_begin, pe = h->hp.cls[c].pair_end;
        if (pe > pb) WB_CUDA(wb::launch_cosx_grad64_class(c, g, pb, pe, h->nsm, s));
    }
    WB_CUDA(wb::launch_grad_rows_sum(gbuf, nblk, natm, grad_out, s));
    return WB_OK;
}

int wb_cosx_g(wb_cosx* h, const double* coords, const double* weights,
              int64_t npts, const float* f, double omega, double tile_tol,
              float* g_out, void* workspace, size_t workspace_bytes,
              void* stream, wb_cosx_stats* stats) {
    if (!h || !f || !g_out || npts <= 0 || !coords || !weights)
        return fail(WB_ERR_INVALID_ARGUMENT, "wb_cosx_g: bad arguments");
    if (!(omega >= 0.0) || !(tile_tol >= 0.0))
        return fail(WB_ERR_INVALID_ARGUMENT, "wb_cosx_g: omega and tile_tol must be >= 0");
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const int64_t ldt = round32(npts);
    const WsLayout L = ws_layout(h, ldt, false);
    if (!workspace || workspace_bytes < L.total)
        return fail(WB_ERR_WORKSPACE, "wb_cosx_g: workspace needs " +
                                          std::to_string(L.total) + " bytes");
    WB_CUDA(cudaMemsetAsync(at<void>(workspace, L.counters), 0,
                            sizeof(unsigned long long) * kCounterWords, s));
    {
        const int st = prepare_omega(h, omega, workspace, L, s);
        if (st != WB_OK) return st;
    }
    int launches = 2;
    int st = tile_prep(h, coords, weights, npts, ldt, f, workspace, L, s, &launches);
    if (st != WB_OK) return st;
    st = run_g_classes(h, npts, ldt, f, g_out, omega, tile_tol, workspace, L, s,
                       &launches);
    if (st != WB_OK) return st;
    return read_stats(h, workspace, L, (ldt / 32) * (int64_t)h->hp.npairs, s,
                      stats, launches);
}

int wb_scf_int1e(wb_cosx* h, int natm, const double* xyz, const double* z,
                 double* s_out, double* t_out, double* v_out, void* stream) {
    if (!h || natm < 0 || (natm && (!xyz || !z)) || !s_out || !t_out || !v_out)
        return fail(WB_ERR_INVALID_ARGUMENT, "wb_scf_int1e: bad arguments");
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    int st = ensure_fp64(h);
    if (st != WB_OK) return st;
    if (natm > h->nuc_cap) {
        WB_CUDA(cudaStreamSynchronize(s));
        if (h->nuc) cudaFree(h->nuc);
        h->nuc = nullptr;
        h->nuc_cap = 0;
        WB_CUDA(cudaMalloc(&h->nuc, sizeof(double) * 4 * (size_t)natm));
        h->nuc_cap = natm;
    }
    if (natm) {
        std::vector<double> nz(4 * (size_t)natm);
        for (int a = 0; a < natm; ++a) {
            for (int x = 0; x < 3; ++x) nz[3 * a + x] = xyz[3 * a + x] - h->origin[x];
            nz[3 * (size_t)natm + a] = z[a];
        }
        WB_CUDA(cudaMemcpyAsync(h->nuc, nz.data(), sizeof(double) * nz.size(),
                                cudaMemcpyHostToDevice, s));
        WB_CUDA(cudaStreamSynchronize(s));     // nz is a host temporary
    }
    wb::scf::Int1eArgs a;
    a.nbas = h->nbas;
    a.nao = h->hp.nao;
    a.sh_l = h->sh_l; a.sh_np = h->sh_np; a.sh_nc = h->sh_nc;
    a.sh_eoff = h->sh_eoff; a.sh_coff = h->sh_coff; a.sh_ao0 = h->sh_ao0;
    a.sh_ctr = h->sh_ctr; a.exps = h->exps; a.coeffs = h->coeffs;
    a.natm = natm;
    a.nuc_xyz = h->nuc;
    a.nuc_z = h->nuc + 3 * (size_t)natm;
    a.boys = h->f64_boys;
    a.S = s_out; a.T = t_out; a.V = v_out;
    WB_CUDA(wb::scf::launch_int1e(a, s));
    return WB_OK;
}

size_t wb_hartree_workspace_bytes(const wb_cosx* h, int64_t npts) {
    if (!h || npts < 0) return 0;
    return hartree_layout(h, npts, hartree_ndh(h->hp)).total;
}

int wb_hartree(wb_cosx* h, const double* coords, int64_t npts, const double* dm,
               double tol, int fp64, double* v_out, void* workspace,
               size_t workspace_bytes, void* stream, int64_t* tasks_kept) {
    if (!h || npts <= 0 || !coords || !dm || !v_out || !(tol >= 0.0))
        return fail(WB_ERR_INVALID_ARGUMENT, "wb_hartree: bad arguments");
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    int st = ensure_fp64(h);
    if (st != WB_OK) return st;
    if ((st = ensure_hartree(h)) != WB_OK) return st;
    const HartreeLayout L = hartree_layout(h, npts, h->ndh);
    if (!workspace || workspace_bytes < L.total)
        return fail(WB_ERR_WORKSPACE, "wb_hartree: workspace needs " +
                                          std::to_string(L.total) + " bytes");
    WB_CUDA(cudaMemsetAsync(at<void>(workspace, L.counters), 0, 256, s));
    wb::scf::DhArgs d;
    std::memset(&d, 0, sizeof(d));
    d.npairs = h->hp.npairs;
    d.nao = h->hp.nao;
    d.D = dm;
    d.hdr = h->hdr;
    d.pclass = h->pclass;
    d.pcls_l = h->pclass;
    d.E = h->f64_E;
    for (int c = 0; c < wb::NCLASS; ++c) {
        d.e_base[c] = h->f64_ebase[c];
        d.pp_begin[c] = h->hp.cls[c].pp_begin;
    }
    d.pref = h->pref;
    d.dh_off = h->dh_off;
    d.dh64 = at<double>(workspace, L.dh64);
    d.dh32 = at<float>(workspace, L.dh32);
    d.pair_dabs = at<float>(workspace, L.dabs);
    WB_CUDA(wb::scf::launch_dh(d, s));
    const int nblk = (int)((npts + 31) / 32);
    WB_CUDA(wb::scf::launch_block_geom(coords, npts, nblk, at<float4>(workspace, L.cr), s));
    wb::scf::HartreeArgs a;
    std::memset(&a, 0, sizeof(a));
    a.coords = coords;
    a.npts = npts;
    a.blk_cr = at<float4>(workspace, L.cr);
    a.nblk = nblk;
    a.npairs = h->hp.npairs;
    a.hdr = h->hdr;
    a.pair_L = h->pair_L;
    a.ptau = h->ptau;
    a.bnd = h->bnd;
    a.bpref = h->bpref;
    a.pair_dabs = d.pair_dabs;
    a.P = h->f64_P;
    a.p = h->p;
    a.geo = h->geo;
    a.p32 = h->p32;
    a.dh_off = h->dh_off;
    a.dh64 = d.dh64;
    a.dh32 = d.dh32;
    a.boys32 = h->boys;
    a.boys64 = h->f64_boys;
    a.tol = tol > 0.0 ? (float)(tol / 1.001) : 0.0f;
    if (tol > 0.0 && a.tol <= 0.0f) a.tol = 1e-38f;
    a.v = v_out;
    a.work = at<int>(workspace, L.counters);
    a.kept = at<unsigned long long>(workspace, L.counters + 64);
    WB_CUDA(wb::scf::launch_hartree(a, fp64 != 0, s));
    if (tasks_kept) {
        unsigned long long kept = 0;
        WB_CUDA(cudaMemcpyAsync(&kept, a.kept, sizeof(kept), cudaMemcpyDeviceToHost, s));
        WB_CUDA(cudaStreamSynchronize(s));
        *tasks_kept = (int64_t)kept;
    }
    return WB_OK;
}

int wb_cosx_screen_mask(wb_cosx* h, const double* coords, const double* weights,
                        int64_t npts, const float* f, double tile_tol, int level,
                        unsigned char* keep, void* workspace,
                        size_t workspace_bytes, void* stream) {
    if (!h || !f || !keep || npts <= 0 || !coords || !weights || level < 0 ||
        level > 2)
        return fail(WB_ERR_INVALID_ARGUMENT, "wb_cosx_screen_mask: bad arguments");
    if (!(tile_tol >= 0.0))
        return fail(WB_ERR_INVALID_ARGUMENT, "wb_cosx_screen_mask: tile_tol must be >= 0");
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const int64_t ldt = round32(npts);
    const WsLayout L = ws_layout(h, ldt, false);
    if (!workspace || workspace_bytes < L.total)
        return fail(WB_ERR_WORKSPACE, "wb_cosx_screen_mask: workspace needs " +
                                          std::to_string(L.total) + " bytes");
    int launches = 0;
    int st = tile_prep(h, coords, weights, npts, ldt, f, workspace, L, s, &launches);
    if (st != WB_OK) return st;
    const wb::CosxArgs a = make_args(h, workspace, L, ldt, npts, f, tile_tol);
    WB_CUDA(wb::launch_screen_mask(a, level, h->hp.npairs, keep, s));
    return WB_OK;
}

int wb_cosx_g_multi(wb_cosx* h, const double* coords, const double* weights,
                    int64_t npts, const float* f, int nomega,
                    const double* omegas, double tile_tol, float* g_out,
                    void* workspace, size_t workspace_bytes, void* stream,
                    wb_cosx_stats* stats) {
    if (!h || !f || !g_out || npts <= 0 || !coords || !weights || nomega < 1 ||
        !omegas)
        return fail(WB_ERR_INVALID_ARGUMENT, "wb_cosx_g_multi: bad arguments");
    for (int j = 0; j < nomega; ++j)
        if (!(omegas[j] >= 0.0))
            return fail(WB_ERR_INVALID_ARGUMENT, "wb_cosx_g_multi: omega must be >= 0");
    if (!(tile_tol >= 0.0))
        return fail(WB_ERR_INVALID_ARGUMENT, "wb_cosx_g_multi: tile_tol must be >= 0");
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const int64_t ldt = round32(npts);
    const WsLayout L = ws_layout(h, ldt, false);
    if (!workspace || workspace_bytes < L.total)
        return fail(WB_ERR_WORKSPACE, "wb_cosx_g_multi: workspace needs " +
                                          std::to_string(L.total) + " bytes");
    WB_CUDA(cudaMemsetAsync(at<void>(workspace, L.counters), 0,
                            sizeof(unsigned long long) * kCounterWords, s));
    int launches = 1;
    int st = tile_prep(h, coords, weights, npts, ldt, f, workspace, L, s, &launches);
    if (st != WB_OK) return st;
    const size_t gsz = (size_t)h->hp.nao * ldt;
    int64_t ntasks = 0;
    // the omega loop of wb_cosx_get_k_multi: a dual pass per omega pair
    for (int j = 0; j < nomega;) {
        if (h->dual_ok && j + 1 < nomega) {
            int ja = j, jb = j + 1;
            if (omegas[jb] < omegas[ja]) std::swap(ja, jb);
            if ((st = prepare_omega_dual(h, omegas[ja], omegas[jb], workspace, L,
                                         s)) != WB_OK)
                return st;
            launches += 3;
            if ((st = run_g_classes_dual(h, npts, ldt, f, g_out + gsz * ja,
                                         g_out + gsz * jb, omegas[ja], omegas[jb],
                                         tile_tol, workspace, L, s, &launches)) != WB_OK)
                return st;
            ntasks += 2 * (ldt / 32) * (int64_t)h->hp.npairs;
            j += 2;
            continue;
        }
        if ((st = prepare_omega(h, omegas[j], workspace, L, s)) != WB_OK) return st;
        launches += 2;
        if ((st = run_g_classes(h, npts, ldt, f, g_out + gsz * j, omegas[j], tile_tol,
                                workspace, L, s, &launches)) != WB_OK)
            return st;
        ntasks += (ldt / 32) * (int64_t)h->hp.npairs;
        j += 1;
    }
    return read_stats(h, workspace, L, ntasks, s, stats, launches);
}

size_t wb_ozaki_workspace_bytes(int nao, int64_t ld) {
    if (nao <= 0 || ld <= 0) return 0;
    return std::max(wb::ozaki_f_bytes(nao, ld), wb::ozaki_k_bytes(nao, ld));
}

int wb_cosx_ozaki_f(wb_cosx* h, const double* x, const double* qd,
                    int64_t ld, float* f_out, void* workspace,
                    size_t workspace_bytes, void* stream) {
    if (!h || !x || !qd || !f_out || ld <= 0 || ld % 32)
        return fail(WB_ERR_INVALID_ARGUMENT, "wb_cosx_ozaki_f: bad arguments");
    const int nao = h->hp.nao;
    if (!wb::ozaki_f_supported(nao))
        return fail(WB_ERR_UNSUPPORTED, "wb_cosx_ozaki_f: nao too large for one "
                                        "exact FP32 level sum");
    if (!workspace || workspace_bytes < wb::ozaki_f_bytes(nao, ld))
        return fail(WB_ERR_WORKSPACE, "wb_cosx_ozaki_f: workspace too small");
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    WB_CUBLAS(cublasSetStream(h->cublas, s));
    WB_CUBLAS(cublasSetMathMode(h->cublas, CUBLAS_DEFAULT_MATH));
    const int r = wb::ozaki_f_gemm(h->cublas, x, qd, nao, ld, f_out, workspace, s);
    if (r) return fail(r >= 1000 ? WB_ERR_CUBLAS : WB_ERR_CUDA,
                       "ozaki F GEMM failed, code " + std::to_string(r));
    return WB_OK;
}

int wb_cosx_ozaki_f64(wb_cosx* h, const double* x, const double* qd,
                      int64_t ld, double* f_out, void* workspace,
                      size_t workspace_bytes, void* stream) {
    if (!h || !x || !qd || !f_out || ld <= 0 || ld % 32)
        return fail(WB_ERR_INVALID_ARGUMENT, "wb_cosx_ozaki_f64: bad arguments");
    const int nao = h->hp.nao;
    if (!wb::ozaki_f_supported(nao))
        return fail(WB_ERR_UNSUPPORTED, "wb_cosx_ozaki_f64: nao too large for one "
                                        "exact FP32 level sum");
    if (!workspace || workspace_bytes < wb::ozaki_f_bytes(nao, ld))
        return fail(WB_ERR_WORKSPACE, "wb_cosx_ozaki_f64: workspace too small");
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    WB_CUBLAS(cublasSetStream(h->cublas, s));
    WB_CUBLAS(cublasSetMathMode(h->cublas, CUBLAS_DEFAULT_MATH));
    const int r = wb::ozaki_f_gemm64(h->cublas, x, qd, nao, ld, f_out, workspace, s);
    if (r) return fail(r >= 1000 ? WB_ERR_CUBLAS : WB_ERR_CUDA,
                       "ozaki F64 GEMM failed, code " + std::to_string(r));
    return WB_OK;
}

int wb_cosx_ozaki_k64(wb_cosx* h, const double* x, const double* g,
                      const double* weights, int64_t npts, int accumulate,
                      double* k_out, void* workspace, size_t workspace_bytes,
                      void* stream) {
    if (!h || !x || !g || !weights || !k_out || npts <= 0)
        return fail(WB_ERR_INVALID_ARGUMENT, "wb_cosx_ozaki_k64: bad arguments");
    const int nao = h->hp.nao;
    const int64_t ld = round32(npts);
    if (!workspace || workspace_bytes < wb::ozaki_k_bytes(nao, ld))
        return fail(WB_ERR_WORKSPACE, "wb_cosx_ozaki_k64: workspace too small");
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    WB_CUBLAS(cublasSetStream(h->cublas, s));
    WB_CUBLAS(cublasSetMathMode(h->cublas, CUBLAS_DEFAULT_MATH));
    const int r = wb::ozaki_k_gemm64(h->cublas, x, g, weights, nao, ld, npts,
                                     accumulate, k_out, workspace, s);
    if (r) return fail(r >= 1000 ? WB_ERR_CUBLAS : WB_ERR_CUDA,
                       "ozaki K64 GEMM failed, code " + std::to_string(r));
    return WB_OK;
}

int wb_ozaki_set_f_engine(int engine) {
    if (engine != WB_OZAKI_ENGINE_LIBRARY && engine != WB_OZAKI_ENGINE_TC)
        return fail(WB_ERR_INVALID_ARGUMENT, "wb_ozaki_set_f_engine: unknown engine");
    wb::ozaki_set_f_engine(engine == WB_OZAKI_ENGINE_TC ? wb::kOzEngineTc
                                                        : wb::kOzEngineLibrary);
    return WB_OK;
}

int wb_ozaki_get_f_engine(void) {
    return wb::ozaki_get_f_engine() == wb::kOzEngineTc ? WB_OZAKI_ENGINE_TC
                                                       : WB_OZAKI_ENGINE_LIBRARY;
}

int wb_cosx_ozaki_k(wb_cosx* h, const double* x, const float* g,
                    const double* weights, int64_t npts, int accumulate,
                    double* k_out, void* workspace, size_t workspace_bytes,
                    void* stream) {
    if (!h || !x || !g || !weights || !k_out || npts <= 0)
        return fail(WB_ERR_INVALID_ARGUMENT, "wb_cosx_ozaki_k: bad arguments");
    const int nao = h->hp.nao;
    const int64_t ld = round32(npts);
    if (!workspace || workspace_bytes < wb::ozaki_k_bytes(nao, ld))
        return fail(WB_ERR_WORKSPACE, "wb_cosx_ozaki_k: workspace too small");
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    WB_CUBLAS(cublasSetStream(h->cublas, s));
    WB_CUBLAS(cublasSetMathMode(h->cublas, CUBLAS_DEFAULT_MATH));
    const int r = wb::ozaki_k_gemm(h->cublas, x, g, weights, nao, ld, npts,
                                   accumulate, k_out, workspace, s);
    if (r) return fail(r >= 1000 ? WB_ERR_CUBLAS : WB_ERR_CUDA,
                       "ozaki K GEMM failed, code " + std::to_string(r));
    return WB_OK;
}

int wb_ao_eval(const wb_cosx* h, const double* coords, int64_t npts,
               double* x_out, void* stream) {
    if (!h || !x_out || npts < 0 || (npts && !coords))
        return fail(WB_ERR_INVALID_ARGUMENT, "wb_ao_eval: bad arguments");
    wb::AoArgs ao;
    ao.coords = coords; ao.npts = npts; ao.ld = round32(npts); ao.nbas = h->nbas;
    ao.sh_l = h->sh_l; ao.sh_np = h->sh_np; ao.sh_nc = h->sh_nc;
    ao.sh_eoff = h->sh_eoff; ao.sh_coff = h->sh_coff; ao.sh_ao0 = h->sh_ao0;
    ao.sh_ctr = h->sh_ctr; ao.exps = h->exps; ao.coeffs = h->coeffs; ao.X = x_out;
    ao.nao = h->hp.nao;
    WB_CUDA(wb::launch_ao_eval(ao, static_cast<cudaStream_t>(stream)));
    return WB_OK;
}

int wb_ao_eval_deriv1(const wb_cosx* h, const double* coords, int64_t npts,
                      double* x_out, void* stream) {
    if (!h || !x_out || npts < 0 || (npts && !coords))
        return fail(WB_ERR_INVALID_ARGUMENT, "wb_ao_eval_deriv1: bad arguments");
    wb::AoArgs ao;
    ao.coords = coords; ao.npts = npts; ao.ld = round32(npts); ao.nbas = h->nbas;
    ao.sh_l = h->sh_l; ao.sh_np = h->sh_np; ao.sh_nc = h->sh_nc;
    ao.sh_eoff = h->sh_eoff; ao.sh_coff = h->sh_coff; ao.sh_ao0 = h->sh_ao0;
    ao.sh_ctr = h->sh_ctr; ao.exps = h->exps; ao.coeffs = h->coeffs; ao.X = x_out;
    ao.nao = h->hp.nao;
    WB_CUDA(wb::launch_ao_eval_d1(ao, static_cast<cudaStream_t>(stream)));
    return WB_OK;
}

int wb_xc_rho(const wb_cosx* h, const double* x, const float* t, int64_t npts,
              int64_t ld, int mgga, double* rho_out, void* stream) {
    if (!h || !x || !t || !rho_out || npts < 0 || ld < npts || ld % 32 != 0)
        return fail(WB_ERR_INVALID_ARGUMENT, "wb_xc_rho: bad arguments");
    WB_CUDA(wb::launch_xc_rho(x, t, h->hp.nao, ld, npts, mgga ? 1 : 0, rho_out,
                              static_cast<cudaStream_t>(stream)));
    return WB_OK;
}

int wb_xc_aow(const wb_cosx* h, const double* x, const double* v, int64_t npts,
              int64_t ld, int mgga, float* g_out, void* stream) {
    if (!h || !x || !v || !g_out || npts < 0 || ld < npts || ld % 32 != 0)
        return fail(WB_ERR_INVALID_ARGUMENT, "wb_xc_aow: bad arguments");
    WB_CUDA(wb::launch_xc_aow(x, v, h->hp.nao, ld, npts, mgga ? 1 : 0, g_out,
                              static_cast<cudaStream_t>(stream)));
    return WB_OK;
}

int wb_int3c1e_dense(const wb_cosx* h, const double* coords, int64_t npts,
                     double omega, float* out, void* stream) {
    if (!h || !out || npts <= 0 || !coords || !(omega >= 0.0))
        return fail(WB_ERR_INVALID_ARGUMENT, "wb_int3c1e_dense: bad arguments");
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const int64_t ldt = round32(npts);
    const size_t om_bytes = align256(sizeof(float) * wb::OMEGA_REC * (size_t)std::max(h->hp.npp, 1));
    const size_t g_bytes = align256(sizeof(float) * 3 * (size_t)ldt);
    void* tmp = nullptr;
    WB_CUDA(cudaMallocAsync(&tmp, om_bytes + 2 * g_bytes, s));
    float4* om = static_cast<float4*>(tmp);
    float* gh = at<float>(tmp, om_bytes);
    float* gl = at<float>(tmp, om_bytes + g_bytes);
    cudaError_t e = wb::launch_omega(h->hp.npp, h->p, h->pref, omega, om, s);
    if (e == cudaSuccess) e = wb::launch_grid_prep(coords, npts, ldt, gh, gl, s);
    if (e == cudaSuccess) {
        e = cudaMemsetAsync(out, 0, sizeof(float) * (size_t)npts * h->hp.nao * h->hp.nao, s);
    }
    if (e == cudaSuccess) {
        wb::CosxArgs a;
        std::memset(&a, 0, sizeof(a));
        a.ld = ldt; a.npts = (int)npts; a.geo = h->geo; a.om = om;
        for (int c = 0; c < wb::NCLASS; ++c) {
            a.Ecls[c] = h->E + h->hp.cls[c].e_base / 4;
            a.pp_begin[c] = h->hp.cls[c].pp_begin;
        }
        a.hdr = h->hdr; a.gxyz_hi = gh; a.gxyz_lo = gl; a.boys = h->boys;
        e = wb::launch_dense_impl(a, h->hp.npairs, h->pclass, h->pl, h->estride,
                                  h->hp.nao, out, s);
    }
    cudaError_t e2 = cudaFreeAsync(tmp, s);
    if (e != cudaSuccess) return cuda_fail(e, "wb_int3c1e_dense");
    if (e2 != cudaSuccess) return cuda_fail(e2, "cudaFreeAsync");
    return WB_OK;
}

int wb_boys_fp32(const float* t, int64_t n, int nmax, float* out,
                 void* stream) {
    if (nmax < 0 || nmax > 6)
        return fail(WB_ERR_INVALID_ARGUMENT, "wb_boys_fp32: nmax must be 0..6");
    if (n < 0 || (n && (!t || !out)))
        return fail(WB_ERR_INVALID_ARGUMENT, "wb_boys_fp32: bad arguments");
    int dev = 0;
    WB_CUDA(cudaGetDevice(&dev));
    float4* tab = nullptr;
    int st = device_boys(dev, &tab);
    if (st != WB_OK) return st;
    WB_CUDA(wb::launch_boys(t, n, nmax, tab, out, static_cast<cudaStream_t>(stream)));
    return WB_OK;
}

int wb_vv10_kernel_sum(const float* xyz, const float* q, const float* w0,
                       const float* kappa, int64_t n, double tile_tol,
                       double* f_out, double* u_out, double* w_out,
                       void* stream, int64_t* pairs_kept) {
    if (n < 0 || !(tile_tol >= 0.0))
        return fail(WB_ERR_INVALID_ARGUMENT, "wb_vv10_kernel_sum: bad arguments");
    if (n && (!xyz || !q || !w0 || !kappa || !f_out || !u_out || !w_out))
        return fail(WB_ERR_INVALID_ARGUMENT, "wb_vv10_kernel_sum: null pointer");
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    if (n == 0) {
        if (pairs_kept) *pairs_kept = 0;
        return WB_OK;
    }
    void* ws = nullptr;
    WB_CUDA(cudaMallocAsync(&ws, wb::vv10_workspace_bytes(n), s));
    cudaError_t e = wb::launch_vv10(xyz, q, w0, kappa, n, tile_tol, f_out,
                                    u_out, w_out, ws, s);
    unsigned long long kept = 0;
    if (e == cudaSuccess && pairs_kept)
        e = cudaMemcpyAsync(&kept, ws, sizeof(kept), cudaMemcpyDeviceToHost, s);
    cudaError_t e2 = cudaFreeAsync(ws, s);
    if (e == cudaSuccess && pairs_kept) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return cuda_fail(e, "wb_vv10_kernel_sum");
    if (e2 != cudaSuccess) return cuda_fail(e2, "cudaFreeAsync");
    if (pairs_kept) *pairs_kept = (int64_t)kept;
    return WB_OK;
}

int wb_vv10_kernel_sum_batch(int nmol, const int64_t* offsets, const float* xyz,
                             const float* q, const float* w0, const float* kappa,
                             double tile_tol, double* f_out, double* u_out,
                             double* w_out, void* stream, int64_t* pairs_kept) {
    if (nmol < 1 || !offsets || !(tile_tol >= 0.0) || offsets[0] != 0)
        return fail(WB_ERR_INVALID_ARGUMENT, "wb_vv10_kernel_sum_batch: bad arguments");
    for (int m = 0; m < nmol; ++m)
        if (offsets[m + 1] < offsets[m])
            return fail(WB_ERR_INVALID_ARGUMENT,
                        "wb_vv10_kernel_sum_batch: offsets must not decrease");
    const int64_t n = offsets[nmol];
    if (n && (!xyz || !q || !w0 || !kappa || !f_out || !u_out || !w_out))
        return fail(WB_ERR_INVALID_ARGUMENT, "wb_vv10_kernel_sum_batch: null pointer");
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    // tiles of 256 points inside each molecule
    std::vector<long long> tstart;
    std::vector<int> tlen, tmol, mtile(nmol + 1, 0);
    for (int m = 0; m < nmol; ++m) {
        mtile[m] = (int)tstart.size();
        for (int64_t i = offsets[m]; i < offsets[m + 1]; i += 256) {
            tstart.push_back(i);
            tlen.push_back((int)std::min<int64_t>(256, offsets[m + 1] - i));
            tmol.push_back(m);
        }
    }
    const int64_t nt = (int64_t)tstart.size();
    mtile[nmol] = (int)nt;
    if (nt > INT32_MAX / 2)
        return fail(WB_ERR_UNSUPPORTED, "wb_vv10_kernel_sum_batch: too many tiles");
    if (nt == 0) {
        if (pairs_kept) *pairs_kept = 0;
        return WB_OK;
    }
    const size_t b_start = align256(sizeof(long long) * nt);
    const size_t b_len = align256(sizeof(int) * nt);
    const size_t b_mol = align256(sizeof(int) * nt);
    const size_t b_mt = align256(sizeof(int) * (nmol + 1));
    const size_t b_st = align256(wb::vv10_tile_stats_bytes(nt));
    char* ws = nullptr;
    WB_CUDA(cudaMallocAsync(reinterpret_cast<void**>(&ws),
                            256 + b_start + b_len + b_mol + b_mt + b_st, s));
    unsigned long long* kept = reinterpret_cast<unsigned long long*>(ws);
    wb::VvSeg sg;
    char* p = ws + 256;
    sg.tstart = reinterpret_cast<const long long*>(p); p += b_start;
    sg.tlen = reinterpret_cast<const int*>(p); p += b_len;
    sg.tmol = reinterpret_cast<const int*>(p); p += b_mol;
    sg.mtile = reinterpret_cast<const int*>(p); p += b_mt;
    void* stats = p;
    sg.ntiles = nt;
    cudaError_t e = cudaMemsetAsync(kept, 0, sizeof(unsigned long long), s);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(const_cast<long long*>(sg.tstart), tstart.data(),
                            sizeof(long long) * nt, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(const_cast<int*>(sg.tlen), tlen.data(), sizeof(int) * nt,
                            cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(const_cast<int*>(sg.tmol), tmol.data(), sizeof(int) * nt,
                            cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(const_cast<int*>(sg.mtile), mtile.data(),
                            sizeof(int) * (nmol + 1), cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess)
        e = wb::launch_vv10_seg(xyz, q, w0, kappa, sg, tile_tol, f_out, u_out, w_out,
                                stats, kept, s);
    unsigned long long kept_h = 0;
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(&kept_h, kept, sizeof(kept_h), cudaMemcpyDeviceToHost, s);
    // the host tables must outlive the copies that read them
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    cudaError_t e2 = cudaFreeAsync(ws, s);
    if (e != cudaSuccess) return cuda_fail(e, "wb_vv10_kernel_sum_batch");
    if (e2 != cudaSuccess) return cuda_fail(e2, "cudaFreeAsync");
    if (pairs_kept) *pairs_kept = (int64_t)kept_h;
    return WB_OK;
}

int wb_fp32_fma_probe(int64_t iters, float* out, int64_t out_len,
                      void* stream, double* flops) {
    int dev = 0, nsm = 1;
    WB_CUDA(cudaGetDevice(&dev));
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    const int threads = 256, blocks = nsm * 8;
    if (!out || out_len < (int64_t)threads * blocks || iters <= 0)
        return fail(WB_ERR_INVALID_ARGUMENT, "wb_fp32_fma_probe: out needs "
                    + std::to_string((int64_t)threads * blocks) + " floats");
    WB_CUDA(wb::launch_fma_probe(iters, blocks, threads, out,
                                 static_cast<cudaStream_t>(stream)));
    if (flops) *flops = 2.0 * 8.0 * 16.0 * (double)iters * threads * blocks;
    return WB_OK;
}

int wb_fp32x2_fma_probe(int64_t iters, float* out, int64_t out_len, void* stream,
                        double* flops) {
    int dev = 0, nsm = 1;
    WB_CUDA(cudaGetDevice(&dev));
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    const int threads = 256, blocks = nsm * 8;
    if (!out || out_len < (int64_t)threads * blocks || iters <= 0)
        return fail(WB_ERR_INVALID_ARGUMENT, "wb_fp32x2_fma_probe: out needs "
                    + std::to_string((int64_t)threads * blocks) + " floats");
    WB_CUDA(wb::launch_fma_probe(iters, blocks, threads, out,
                                 static_cast<cudaStream_t>(stream), true));
    if (flops) *flops = 2.0 * 2.0 * 8.0 * 16.0 * (double)iters * threads * blocks;
    return WB_OK;
}

}  // extern "C"
