// Host-side (FP64) preprocessing of the COSX path: basis, shell pairs,
// Boys table, Becke weights.  Internal header of libwb97mv_gb300.
#pragma once
#include <cstdint>
#include <string>
#include <vector>

#include "wb97mv_gb300.h"

namespace wb {

constexpr int LMAX = 3;
constexpr int NCLASS = 10;          // (la >= lb) classes, la, lb <= 3
constexpr int BOYS_NODES = 145;     // T_k = k / 4, k = 0..144 (T < 36)
constexpr int BOYS_ROW = 20;        // floats per table row (kernel layout)
constexpr int OMEGA_REC = 20;       // floats per primitive pair per omega
constexpr int NIA_MAX = 16;         // functions per shell (reference cap)
constexpr int PPR_MAX = 16;         // primitives per shell (reference cap)

inline int ncart(int l) { return (l + 1) * (l + 2) / 2; }
inline int nsph(int l) { return 2 * l + 1; }
inline int class_of(int la, int lb) { return la * (la + 1) / 2 + lb; }
// packed Hermite coefficients per axis for a (la >= lb) class, E^{00}_0 = 1
// excluded: sum_{i<=la, i'<=lb} (i + i' + 1) - 1
int e_count_axis(int la, int lb);
// floats of E per primitive pair (3 axes, padded to a multiple of 4)
int e_stride(int la, int lb);

void cart_components(int l, std::vector<int>& ix, std::vector<int>& iy,
                     std::vector<int>& iz);
// (ncart, nsph) row-major real-solid-harmonic transform, unit-sphere norm
std::vector<double> cart2sph(int l);
// max over spherical columns of sum_cart |c2s| (screening tau per shell)
double c2s_tau(int l);

// FP64 Boys F_0..F_nmax at T (series + downward recursion below T = 40,
// F_0 from erf plus upward recursion above)
void boys_f64(int nmax, double t, double* out);
// kernel table: BOYS_NODES rows of BOYS_ROW floats
std::vector<float> boys_table();

struct VShell {                     // one contraction column of one shell
    int phys, ci, atom, l, nprim, ao0;
    double A[3];                    // centre relative to the origin
    std::vector<double> exps, coef;
    double cmax;                    // max |coef|
};

struct ClassRange {
    int pair_begin = 0, pair_end = 0;
    int pp_begin = 0, pp_end = 0;
    int64_t e_base = 0;             // float offset of the class's E block
};

struct HostPairs {
    int nao = 0, nbas_phys = 0, nvshell = 0, npairs = 0, npp = 0;
    std::vector<VShell> vsh;
    // per pair (device order: sorted by class)
    std::vector<int32_t> hdr;       // 4 per pair: ia0, ib0, pp0, npp|diag<<16
    // kernel form of hdr: ia0 | ga0 << 16, ib0 | gb0 << 16, pp0, npp|diag<<16
    // with ga0 / gb0 the rows of A / B in the class's partial-G buffer
    std::vector<int32_t> khdr;
    std::vector<int32_t> pshell;    // 2 per pair: vshell A, vshell B
    std::vector<float> ptau;        // 2 per pair: tau, tau * sum(pref)
    std::vector<int32_t> pclass, pish, pjsh;
    std::vector<int64_t> pflops;    // model flops per grid point
    std::vector<int32_t> pnint;     // nfi * nfj
    // per primitive pair
    std::vector<float> geo;         // 8 per pp: P hi (3), 0, P lo (3), 0
    std::vector<double> p, pref;    // exponent sum, folded prefactor
    std::vector<float> bnd;         // 4 per pp: P (3), p' = 0.75 p
    std::vector<float> bpref;       // bound prefactor, rounded up
    std::vector<float> E;           // per class blocks, e_stride per pp
    ClassRange cls[NCLASS];
    // per-class partial G buffers: class (la, lb) holds the AOs of the
    // l = la shells (rows 0 ..) then, for lb != la, those of the l = lb
    // shells, each group in AO order
    int nlao[LMAX + 1] = {0, 0, 0, 0};   // AOs per angular momentum
    int crow[NCLASS] = {0};              // rows of each class buffer
    int64_t crow_base[NCLASS] = {0};     // first row of each class buffer
    int64_t ncrow = 0;                   // rows of all class buffers
    std::vector<int32_t> gsrc;           // 4 per AO: class-buffer rows that
                                         // sum to G, ascending class, -1 pad
    // packed per-class primitive-pair records (geo, omega record, E) that
    // the class kernels read; rebuilt per omega
    int64_t rec_off[NCLASS] = {0};       // float4 offset of each class
    int64_t nrec = 0;                    // float4 in all classes
    int64_t rec_off2[NCLASS] = {0};      // the same for the dual-omega layout
    int64_t nrec2 = 0;
    // per virtual shell (for the sub-block statistics)
    std::vector<int32_t> vs_ao0, vs_nf;
};

// Builds the pair tables; returns WB_OK or an error code with `err` set.
int build_pairs(const wb_basis& b, const double origin[3], double cutoff,
                HostPairs& out, std::string& err);

// FP64 pair data of the plain FP64 G kernels (cosx_fp64.cu), per primitive
// pair in the order of the pair tables: P (3 per pair, molecule frame) and,
// in one block per class, the Hermite E^{i,j}_t of the three axes laid out
// [axis][i][j][t] (i <= la, j <= lb, t <= i + j, E^{00}_0 = 1 included).
int e64_axis(int la, int lb);        // sum_{i <= la, j <= lb} (i + j + 1)
struct HostPairs64 {
    std::vector<double> P;
    std::vector<double> alpha;       // bra (shell A) exponent per primitive pair
    std::vector<double> E;
    int64_t e_base[NCLASS] = {0};    // double offset of each class's E block
};
void build_pairs64(const HostPairs& hp, HostPairs64& out);

// FLOP model of one (bra ish, ket jsh) task per grid point.
int64_t model_flops(int la, int lb, int npi, int npj, bool diag);

void becke_partition(const double* pts, int64_t n, const int* owner,
                     const double* atoms, int natm, double* out);

}  // namespace wb
