/*
 * wb97mv_gb300.h -- C ABI of the GB300 (sm_103a) COSX exchange hot path.
 *
 * Plain C: no CUDA, PyTorch or C++ types cross this boundary.  Device
 * buffers are raw pointers owned by the caller; `stream` is a cudaStream_t
 * passed as void*.  Every entry point returns an int status (0 = WB_OK,
 * > 0 = one of the WB_ERR_* codes below); wb_last_error() holds a one-line
 * description of the last failure on the calling thread.  No C++
 * exception crosses the boundary and nothing falls back to the CPU.
 *
 * Layouts.  Per-grid-point matrices are AO-major: element (mu, g) of X, F
 * and G sits at mu * ldp + g, ldp = npts rounded up to a multiple of 32 (one
 * warp-sized sub-block).  Coordinates are FP64 (npts, 3) row-major, in the
 * frame of the handle's `origin`.  Square AO matrices (QD, K) are
 * (nao, nao) row-major.
 *
 * The reference computes the same quantities in Python/CuPy; each function
 * names the reference interface it replaces (paths inside the reference
 * project Cedrus810/pyscf-wb97mv-fast).
 */
#ifndef WB97MV_GB300_H
#define WB97MV_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* -- status codes --------------------------------------------------------- */
#define WB_OK 0
#define WB_ERR_INVALID_ARGUMENT 1
#define WB_ERR_UNSUPPORTED 2      /* reference: gpu/xc.py:30 Unsupported */
#define WB_ERR_CUDA 3
#define WB_ERR_CUBLAS 4
#define WB_ERR_OUT_OF_MEMORY 5
#define WB_ERR_WORKSPACE 6        /* workspace pointer/size too small */
#define WB_ERR_NO_DEVICE 7

/* Basis description (libcint conventions: per-primitive radial norm folded
 * into the coefficients, contracted functions normalised).  Shell s has
 * nprim exponents at exps[shell_exp_off[s]] and an (nprim, nctr) row-major
 * coefficient block at coeffs[shell_coef_off[s]].  Replaces the Mole
 * accessors read by gpu/shellpairs.py:187-221 and gpu/ao_eval.py:66-111. */
typedef struct wb_basis {
    int natm;
    int nbas;
    const double* atom_coords;   /* (natm, 3) bohr */
    const int* shell_atom;       /* (nbas,) */
    const int* shell_l;          /* (nbas,) 0..3 */
    const int* shell_nprim;      /* (nbas,) */
    const int* shell_nctr;       /* (nbas,) */
    const int* shell_exp_off;    /* (nbas,) */
    const int* shell_coef_off;   /* (nbas,) */
    const double* exps;
    const double* coeffs;
} wb_basis;

/* Counters of one G / K build.  tasks = (32-point sub-block, shell pair);
 * integrals = sum over kept tasks of points * nfi * nfj (the definition of
 * benchmarks/experimental/cosx/cint_shim.c:75-77); model_flops = the
 * algorithmic flop model of kept tasks (pyscf_wb97mv_fast_gb300/
 * flops_model.py).  Mirrors GpuKBuilder.last_stats (gpu/sgx_k.py:743-748). */
typedef struct wb_cosx_stats {
    int64_t tasks_total;
    int64_t tasks_kept;
    double integrals;
    double model_flops;
    int64_t tasks_kept_class[10];
    double model_flops_class[10];
    int32_t kernel_launches;      /* device kernels launched by the call */
    int32_t reserved;
    /* with WB_K_PROFILE: device ms per phase, summed over tiles: AO
     * values, F GEMM, F cast, sub-block stats + G kernels, w o G, K GEMM */
    double phase_ms[6];
} wb_cosx_stats;

typedef struct wb_cosx_info {
    int nao;
    int nbas;                     /* after splitting general contractions */
    int npairs;                   /* kept shell pairs */
    int nprim_pairs;
    int class_pairs[10];          /* pairs per (la >= lb) class */
    int class_prim_pairs[10];
} wb_cosx_info;

typedef struct wb_cosx wb_cosx;   /* opaque per-(molecule, device) handle */

/* Flags of wb_cosx_get_k */
#define WB_K_GEMM_NATIVE_FP64 0   /* cuBLAS DGEMM */
#define WB_K_GEMM_EMULATED_FP64 1 /* cuBLAS FP64 fixed-point emulation */
#define WB_K_GEMM_OZAKI_BF16 2    /* FP64-accurate Ozaki split on bf16
                                     tensor cores (7-bit slices, exact
                                     FP32 level sums, FP64 combination) */
#define WB_K_PROFILE 4            /* record per-phase CUDA events (stats) */

/* Build the packed shell-pair tables of a molecule on the host (FP64) and
 * upload them to the current device.  origin (3,) is subtracted from every
 * centre (the kernels work in a molecule-centred frame).  pair_cutoff is the
 * primitive magnitude cut (1e-14 in the reference).  Replaces
 * ShellPairs.__init__ + to_device (gpu/shellpairs.py:184-437) and
 * GpuKBuilder._build (gpu/sgx_k.py:593-612).  Out-of-scope bases (l > 3,
 * nprim > 16, nctr * (2l+1) > 16, spinor/cartesian) return
 * WB_ERR_UNSUPPORTED. */
int wb_cosx_create(const wb_basis* basis, const double origin[3],
                   double pair_cutoff, wb_cosx** out);
int wb_cosx_destroy(wb_cosx* h);
int wb_cosx_get_info(const wb_cosx* h, wb_cosx_info* info);

/* Host copies of the pair tables, for tests: per pair (ia0, ib0, pp0,
 * npp | diag << 16, class, ish, jsh, model flops per point) as int64 rows of
 * 8; returns the number of rows written (<= cap). */
int64_t wb_cosx_export_pairs(const wb_cosx* h, int64_t* rows, int64_t cap);

/* Bytes of device workspace wb_cosx_get_k / wb_cosx_g need for a grid of
 * npts points processed in tiles of tile_pts points (0 = one tile). */
size_t wb_cosx_workspace_bytes(const wb_cosx* h, int64_t npts,
                               int64_t tile_pts);

/* One full COSX K build on the device:
 *   per tile: X = AO values (FP64)                  gpu/ao_eval.py:186-329
 *             F = fl32(X QD)  (FP64 GEMM)           gpu/sgx_k.py:719-722
 *             sub-block stats + fused screen + G    gpu/sgx_k.py:754-781,
 *               G_gv = sum_mu A^g_mu,v F_g,mu       :866-924, :165-400
 *             K += X^T (w o G)  (FP64 GEMM)         gpu/sgx_k.py:734
 * qd = proj @ dm (nao, nao) row-major, FP64.  k_out (nao, nao) row-major is
 * overwritten with the unsymmetrised K (the caller applies proj^T and
 * (K + K^T)/2, gpu/sgx_k.py:736-742).  tile_tol = 0 keeps every task.
 * Replaces GpuKBuilder.get_k (gpu/sgx_k.py:663-751). */
int wb_cosx_get_k(wb_cosx* h, const double* coords, const double* weights,
                  int64_t npts, const double* qd, double omega,
                  double tile_tol, int64_t tile_pts, int flags,
                  double* k_out, void* workspace, size_t workspace_bytes,
                  void* stream, wb_cosx_stats* stats);

/* wb_cosx_get_k for nomega range-separation parameters and one density:
 * the AO values, F = fl32(X QD) and the block statistics of each tile are
 * formed once and serve every omega; k_out holds nomega (nao, nao)
 * row-major matrices, omega j at k_out + j nao^2, each equal to what
 * wb_cosx_get_k returns for omegas[j].  stats sum over the omegas.  The
 * reference reaches the same pair of matrices (omega = 0 and the
 * functional's omega, one density) through two get_k_only calls of one
 * SCF cycle (gpu/sgx_k.py:983-990, via GpuKBuilder.get_k :663-751). */
int wb_cosx_get_k_multi(wb_cosx* h, const double* coords,
                        const double* weights, int64_t npts, const double* qd,
                        int nomega, const double* omegas, double tile_tol,
                        int64_t tile_pts, int flags, double* k_out,
                        void* workspace, size_t workspace_bytes, void* stream,
                        wb_cosx_stats* stats);

/* COSX exchange nuclear gradient with the grid response off, in FP64:
 * grad_out (natm, 3) = dE/dR of E = -1/4 tr(D K(omega)) at fixed D, fixed
 * grid points and weights (the SGX gradient with grid response off), for
 * the plain SGX K (no PJS projector: dm is the symmetric density).  Two
 * parts: the AO-value side 1/2 sum_g w_g sum_{mu on C} grad X_g,mu (G D)_g,mu
 * with G from the FP64 class kernels, and the integral side
 * -1/2 sum_g w_g sum_{nu on C, lam} F_g,nu F_g,lam d(nu lam|g)/dR_nu from
 * FP64 derivative kernels (d/dA = 2 alpha (a+1) - a_x (a-1); the ket side
 * by translational invariance).  tile_tol screens tasks as the K build
 * does.  Bitwise reproducible.  The reference computes gradients with
 * stock PySCF (pyscf.sgx.grad, grid response off; README.md:134-137) and
 * has no GPU gradient of its own (README.md:168).  Calls the same lazy
 * FP64 table upload as wb_cosx_get_k_fp64. */
size_t wb_cosx_k_grad_workspace_bytes(const wb_cosx* h, int64_t npts, int natm);
int wb_cosx_k_grad(wb_cosx* h, const double* coords, const double* weights,
                   int64_t npts, const double* dm, double omega, double tile_tol,
                   int natm, double* grad_out, void* workspace,
                   size_t workspace_bytes, void* stream);

/* Kernel variant of one class on this handle (the knobs of the autotuner,
 * pyscf_wb97mv_fast_gb300/autotune.py): dual = 1 runs the class's
 * two-omega kernel in two-omega passes (else one single-omega launch per
 * omega); staged = 1 stages each task's primitive-pair records in shared
 * memory (else they are prefetched into registers).  A variant the
 * molecule cannot run (records too large for shared memory, no two-omega
 * kernel) returns WB_ERR_UNSUPPORTED and leaves the class as it was.
 * Results are the same to FP32 rounding whatever the variant; each variant
 * is deterministic.  The reference has one kernel per class
 * (gpu/sgx_k.py:165-400) and no autotuner. */
int wb_cosx_set_class_variant(wb_cosx* h, int cls, int dual, int staged);
int wb_cosx_get_class_variant(const wb_cosx* h, int cls, int* dual, int* staged);

/* Plain FP64 form of the K build: the same steps as wb_cosx_get_k_multi
 * with every step in FP64 and nothing rounded to FP32.  X (FP64 AO values)
 * -> F = X QD (cuBLAS DGEMM, kept FP64) -> the same screen (block
 * statistics of fl32(F), 32-point blocks, tile_tol) -> G by FP64 class
 * kernels (FP64 Boys, McMurchie-Davidson recurrences, Hermite sums and
 * contraction; G accumulated in FP64) -> K = X^T (w o G) (cuBLAS DGEMM).
 * The whole grid is one tile.  k_out holds nomega (nao, nao) row-major
 * unsymmetrised K, as wb_cosx_get_k_multi.  It is the comparison point of
 * the mixed-precision path and an FP64 operator for the SCF tail; the
 * reference's FP64 tail takes the hooks off and runs stock PySCF's
 * get_k_only on the CPU (staging/schedule.py:329-334), so this entry has
 * no GPU counterpart there.  The first call on a handle builds and uploads
 * the FP64 pair tables (synchronous device allocation and copies), so it
 * must not be inside a stream capture.  Workspace:
 * wb_cosx_fp64_workspace_bytes(h, npts) (36 B per point and AO). */
size_t wb_cosx_fp64_workspace_bytes(const wb_cosx* h, int64_t npts);
int wb_cosx_get_k_fp64(wb_cosx* h, const double* coords, const double* weights,
                       int64_t npts, const double* qd, int nomega,
                       const double* omegas, double tile_tol, double* k_out,
                       void* workspace, size_t workspace_bytes, void* stream,
                       wb_cosx_stats* stats);

/* Batched K builds: the K of several molecules per call, with one launch
 * per class kernel over all of them (a class with no two-omega kernel:
 * one per omega).  A plan fixes the molecules (handles, each used by this
 * plan only while it lives), their grids (coords, weights, npts; device
 * memory that must stay unchanged), their workspaces (owned by the plan
 * while it lives), the omegas (1 or 2) and tile_tol.  wb_cosx_batch_create
 * evaluates the AO values, the grid coordinates and the omega records
 * once (on `stream`, synchronised before it returns).  The F / K split
 * scratch is one buffer shared by the molecules (they use it one after
 * another): each molecule's workspace needs wb_cosx_batch_workspace_bytes
 * bytes and the scratch the largest *scratch_bytes it reports.  Each
 * wb_cosx_batch_run takes one density per molecule (qd[m], (nao_m,
 * nao_m) row-major) and writes nomega unsymmetrised K matrices per
 * molecule to k_out[m], as wb_cosx_get_k_multi does (omega j at k_out[m]
 * + j nao_m^2).  qd[m] == NULL leaves molecule m out of this run (its
 * F is zero, so its screen keeps no task; k_out[m] may be NULL and is not
 * written): the molecules of one plan can stand at different SCF stages.
 * At least one molecule must be built.  A run makes no allocation and, with stats == NULL, no
 * host synchronisation, so it can be captured in a CUDA graph.  Each
 * molecule's K equals its wb_cosx_get_k_multi result when the handles
 * agree on the kernel variant of every class (the same elements and
 * basis).  The reference builds one molecule's K per call
 * (GpuKBuilder.get_k, gpu/sgx_k.py:663-751) and has no batched form
 * (batch throughput is a non-goal, docs/design.en.md:44). */
typedef struct wb_cosx_batch wb_cosx_batch;
size_t wb_cosx_batch_workspace_bytes(const wb_cosx* h, int64_t npts,
                                     size_t* scratch_bytes);
int wb_cosx_batch_create(int nmol, wb_cosx* const* handles,
                         const double* const* coords, const double* const* weights,
                         const int64_t* npts, void* const* workspaces,
                         const size_t* workspace_bytes, void* scratch,
                         size_t scratch_bytes, int nomega, const double* omegas,
                         double tile_tol, int flags, void* stream,
                         wb_cosx_batch** out);
int wb_cosx_batch_run(wb_cosx_batch* b, const double* const* qd,
                      double* const* k_out, void* stream, wb_cosx_stats* stats);
int wb_cosx_batch_destroy(wb_cosx_batch* b);

/* The fused G kernels alone on one tile: f (nao, ldp) FP32 AO-major in,
 * g_out (nao, ldp) FP32 out (overwritten).  weights (npts,) FP64 feed the
 * screening estimate.  Replaces GpuKBuilder._tasks + _launch
 * (gpu/sgx_k.py:813-843, :754-781). */
int wb_cosx_g(wb_cosx* h, const double* coords, const double* weights,
              int64_t npts, const float* f, double omega, double tile_tol,
              float* g_out, void* workspace, size_t workspace_bytes,
              void* stream, wb_cosx_stats* stats);

/* One-electron integrals of the handle's basis in FP64 on the device:
 * s_out (overlap), t_out (kinetic energy) and v_out (attraction of natm
 * point charges z[a] at xyz[3a..3a+2], bohr, absolute frame), each
 * (nao, nao) row-major and symmetric.  Same contracted spherical AOs as
 * wb_ao_eval.  xyz and z are host arrays.  The reference's SCF takes these
 * from PySCF on the host (mol.intor('int1e_ovlp' / 'int1e_kin' /
 * 'int1e_nuc') inside scf.hf, below staging/schedule.py:455-485); no
 * reference GPU counterpart. */
int wb_scf_int1e(wb_cosx* h, int natm, const double* xyz, const double* z,
                 double* s_out, double* t_out, double* v_out, void* stream);

/* Bytes of device workspace wb_hartree needs for npts points. */
size_t wb_hartree_workspace_bytes(const wb_cosx* h, int64_t npts);

/* Hartree potential of a density at grid points:
 *   v_out[g] = sum_{mu nu} D_{mu nu} (mu nu | 1/|r - r_g|)
 * coords (npts, 3) FP64 device (the handle frame, like wb_cosx_get_k), dm
 * (nao, nao) FP64 device, symmetric.  Per iteration a Hermite density of
 * every primitive pair is formed from dm; one warp per 32-point block then
 * sums the pairs that pass the COSX kernels' locked bound times
 * (2 - delta_AB) sum |D_AB| >= tol (0 keeps every pair).  fp64 = 1: FP64
 * throughout; 0: FP32 Boys, recurrence and sums over 32-pair chunks, FP64
 * across chunks.  Bitwise reproducible.  *tasks_kept (if not null, a
 * synchronisation) receives the kept (block, pair) count.  With
 * J = X^T (w o v) X it is the SCF's Coulomb matrix on the SGX grid (the
 * reference's SCF gets J from PySCF's SGX get_jk, core/sgx_patch.py:33-53). */
int wb_hartree(wb_cosx* h, const double* coords, int64_t npts, const double* dm,
               double tol, int fp64, double* v_out, void* workspace,
               size_t workspace_bytes, void* stream, int64_t* tasks_kept);

/* The fused screen of the G kernels alone, as a mask: keep (nblk, npairs)
 * uint8 on the device, row-major, 1 where the class kernels keep task
 * (point block, pair) at tile_tol.  Blocks hold 32 << level points (level
 * 0, 1, 2; nblk = ceil(round32(npts) / (32 << level))); pair k is row k of
 * wb_cosx_export_pairs.  Same block statistics, pair bound data and screen
 * function as wb_cosx_g; same workspace.  A test aid: replaces the device
 * keep mask (_keep_mask_device, gpu/sgx_k.py:866-903) that the
 * reference's superset test reads (tests/gpu/test_sgx_k.py:166-206). */
int wb_cosx_screen_mask(wb_cosx* h, const double* coords, const double* weights,
                        int64_t npts, const float* f, double tile_tol, int level,
                        unsigned char* keep, void* workspace,
                        size_t workspace_bytes, void* stream);

/* wb_cosx_g for nomega omegas and one F: the block statistics are formed
 * once, and omegas are taken in pairs by the two-omega class kernels (one
 * screen, F loads and distances per pair of omegas), as in
 * wb_cosx_get_k_multi.  g_out holds nomega (nao, ldp) FP32 arrays, omega j
 * at g_out + j nao ldp, each equal to what wb_cosx_g returns for
 * omegas[j].  Same workspace as wb_cosx_g.  Replaces the _tasks + _launch
 * part (gpu/sgx_k.py:754-781, :813-843) of the reference's two K builds of
 * one SCF cycle. */
int wb_cosx_g_multi(wb_cosx* h, const double* coords, const double* weights,
                    int64_t npts, const float* f, int nomega,
                    const double* omegas, double tile_tol, float* g_out,
                    void* workspace, size_t workspace_bytes, void* stream,
                    wb_cosx_stats* stats);

/* The two FP64-accurate GEMMs of the K build on the bf16 tensor cores
 * (Ozaki split, WB_K_GEMM_OZAKI_BF16), callable alone:
 *   wb_cosx_ozaki_f: f_out (nao, ld) FP32 = fl32(X QD), x (nao, ld) FP64
 *     AO-major, qd (nao, nao) row-major; needs 7 nao < 16384.
 *     Replaces F = (X @ proj_dm).astype(float32) (gpu/sgx_k.py:722).
 *   wb_cosx_ozaki_k: k_out (nao, nao) row-major (+)= X^T (w o G) over npts
 *     points, g (nao, ld) FP32.  Replaces K += X.T @ (w64 * G)
 *     (gpu/sgx_k.py:734).
 * Workspace: wb_ozaki_workspace_bytes(nao, ld) bytes. */
size_t wb_ozaki_workspace_bytes(int nao, int64_t ld);
int wb_cosx_ozaki_f(wb_cosx* h, const double* x, const double* qd,
                    int64_t ld, float* f_out, void* workspace,
                    size_t workspace_bytes, void* stream);
int wb_cosx_ozaki_k(wb_cosx* h, const double* x, const float* g,
                    const double* weights, int64_t npts, int accumulate,
                    double* k_out, void* workspace, size_t workspace_bytes,
                    void* stream);

/* The same two products with FP64 operands on the output / G side, for
 * the SCF's FP64 tail (the reference's FP64 numint GEMMs, gpu/xc.py:130-201
 * and gpu/vv10.py:288-297, run there in FP64):
 *   wb_cosx_ozaki_f64: f_out (nao, ld) FP64 = X QD, the combined 42-bit
 *     level sums rounded once to FP64;
 *   wb_cosx_ozaki_k64: k_out (+)= X^T (w o G) with g (nao, ld) FP64.
 * Same workspace and limits as wb_cosx_ozaki_f / wb_cosx_ozaki_k. */
int wb_cosx_ozaki_f64(wb_cosx* h, const double* x, const double* qd,
                      int64_t ld, double* f_out, void* workspace,
                      size_t workspace_bytes, void* stream);
int wb_cosx_ozaki_k64(wb_cosx* h, const double* x, const double* g,
                      const double* weights, int64_t npts, int accumulate,
                      double* k_out, void* workspace, size_t workspace_bytes,
                      void* stream);

/* Engine of the F product (process-wide, every F of the K builds and of
 * wb_cosx_ozaki_f / _f64): WB_OZAKI_ENGINE_LIBRARY (the default) runs one
 * cuBLAS bf16 GEMM per level; WB_OZAKI_ENGINE_TC is this library's
 * tensor-core kernel (TMA tile loads, tcgen05 MMAs into TMEM, the exact
 * level combination fused into its epilogue), slower on the bench step
 * (its seven level accumulators allow 64-wide tiles only).  Both give
 * bitwise the same F.  Replaces
 * no reference call (the reference's F GEMM is one CuPy FP64 matmul,
 * gpu/sgx_k.py:722); returns WB_OK or WB_ERR_INVALID_ARGUMENT. */
#define WB_OZAKI_ENGINE_LIBRARY 0
#define WB_OZAKI_ENGINE_TC 1
int wb_ozaki_set_f_engine(int engine);
int wb_ozaki_get_f_engine(void);

/* AO values X (nao, ldp) FP64 AO-major at npts points (FP64 arithmetic).
 * Replaces AoEvaluator.eval(deriv=0) with dtype FP64 (gpu/ao_eval.py:186-329). */
int wb_ao_eval(const wb_cosx* h, const double* coords, int64_t npts,
               double* x_out, void* stream);

/* AO values and their x, y, z gradients, x_out (4, nao, ldp) FP64.
 * Replaces AoEvaluator.eval(deriv=1) (gpu/ao_eval.py:186-329) for the VV10
 * flow (gpu/vv10.py:288-297). */
int wb_ao_eval_deriv1(const wb_cosx* h, const double* coords, int64_t npts,
                      double* x_out, void* stream);

/* Semilocal XC flow (NumInt.nr_rks for one RKS density; the reference's
 * gpu_nr_rks, gpu/xc.py:130-201), the two pointwise passes around the host
 * functional.  x (4, nao, ld) FP64 from wb_ao_eval_deriv1; ld a multiple of
 * 32 and >= npts.
 *   wb_xc_rho: t (1 or 4, nao, ld) FP32 = fl32(dm^T x_d) (wb_cosx_ozaki_f on
 *     each plane; plane 0 only unless mgga); rho_out (5, ld) FP64 = (rho,
 *     grad x/y/z, tau) -- gpu/xc.py:158-172.
 *   wb_xc_aow: v (5, ld) FP64, the density-parameter derivatives (chain
 *     rule applied, gpu/xc.py:96-116); g_out (1 or 4, nao, ld) FP32: plane 0
 *     = 1/2 v0 x0 + sum_d v_d x_d, planes 1..3 (mgga) = 1/2 vtau x_d.  Then
 *     vmat = K + K^T + sum_d K_d with K = wb_cosx_ozaki_k(x0, plane 0, w)
 *     and K_d = wb_cosx_ozaki_k(x_d, plane d, w) -- gpu/xc.py:179-201.
 * Points at or past npts get 0 in both. */
int wb_xc_rho(const wb_cosx* h, const double* x, const float* t, int64_t npts,
              int64_t ld, int mgga, double* rho_out, void* stream);
int wb_xc_aow(const wb_cosx* h, const double* x, const double* v, int64_t npts,
              int64_t ld, int mgga, float* g_out, void* stream);

/* Dense contracted spherical A[g, mu, nu] (npts, nao, nao) FP32 for small
 * validation systems.  Replaces int3c1e_fp32 (gpu/int3c1e.py:284-314). */
int wb_int3c1e_dense(const wb_cosx* h, const double* coords, int64_t npts,
                     double omega, float* out, void* stream);

/* FP32 Boys F_0..F_nmax (nmax <= 6) of n arguments: out (nmax+1, n).
 * Replaces boys_eval (gpu/boys.py:194-204). */
int wb_boys_fp32(const float* t, int64_t n, int nmax, float* out,
                 void* stream);

/* Host FP64 Boys F_0..F_nmax at one argument (used to build the table). */
int wb_boys_f64_host(int nmax, double t, double* out);

/* Host only (no device): model flops per grid point summed over the shell
 * pairs the COSX kernels keep for this basis -- the reference's pair
 * enumeration and magnitude cut (gpu/shellpairs.py:287-294) and the flop
 * model of the G kernels, i.e. the work of one grid point with no task
 * screening.  npairs_out (may be NULL) receives the number of pairs. */
int wb_model_flops_per_point(const wb_basis* basis, double pair_cutoff,
                             double* flops_out, int64_t* npairs_out);

/* VV10 double sum over n points (FP32 pair terms, FP64 per-point sums):
 *   F_i = -1.5 sum_j q_j / (g gp (g + gp)),  U_i = sum_j T (1/g + 1/(g+gp)),
 *   W_i = sum_j T (1/g + 1/(g+gp)) R^2,  g = R^2 w0_i + kappa_i, gp likewise.
 * xyz (n, 3), q, w0, kappa (n,) FP32; F, U, W (n,) FP64.  Tile pairs whose
 * bound is below tile_tol are skipped (0 keeps every pair).
 * Replaces Vv10Kernel.kernel_sum (gpu/vv10.py:167-240). */
int wb_vv10_kernel_sum(const float* xyz, const float* q, const float* w0,
                       const float* kappa, int64_t n, double tile_tol,
                       double* f_out, double* u_out, double* w_out,
                       void* stream, int64_t* pairs_kept);

/* wb_vv10_kernel_sum for several molecules in one launch: the points of
 * molecule m are offsets[m] .. offsets[m + 1] - 1 of the concatenated
 * arrays (offsets: nmol + 1 host int64, offsets[0] = 0), and each point's
 * double sum runs over its own molecule's points only.  Every molecule's
 * F, U, W are bitwise what wb_vv10_kernel_sum returns for it alone.
 * *pairs_kept sums over the molecules.  Synchronises `stream` before it
 * returns (the host tile tables are copied).  The reference sums one
 * molecule per call (Vv10Kernel.kernel_sum, gpu/vv10.py:167-240). */
int wb_vv10_kernel_sum_batch(int nmol, const int64_t* offsets, const float* xyz,
                             const float* q, const float* w0, const float* kappa,
                             double tile_tol, double* f_out, double* u_out,
                             double* w_out, void* stream, int64_t* pairs_kept);

/* Allocation-free VV10 double sum: the same computation and results as
 * wb_vv10_kernel_sum, for callers that cannot let the library allocate
 * device memory (e.g. a host framework that reserves the whole GPU memory
 * up front and hands out fixed arenas, where a cudaMalloc during a request
 * would fail or stall the device).  Its scratch (tile statistics and the
 * kept-pair counter) is a file-scope device array of fixed size, held by
 * every GPU that loads the library until the process exits; n above
 * WB_VV10_NOALLOC_MAX_POINTS is rejected with WB_ERR_INVALID_ARGUMENT.
 * Each call looks up the array's device address in the current context
 * (cudaGetSymbolAddress, no allocation), so a context torn down and made
 * again is served; make the first call on a device before any stream
 * capture (it may load the library's module into the context).
 * All calls on a device share the array and
 * each call leaves its own contents there: calls whose work overlaps on
 * the GPU (different streams, or different host threads) race.  No
 * counterpart in the reference. */
#define WB_VV10_NOALLOC_MAX_POINTS 1048576
int wb_vv10_kernel_sum_noalloc(const float* xyz, const float* q,
                               const float* w0, const float* kappa,
                               int64_t n, double tile_tol, double* f_out,
                               double* u_out, double* w_out, void* stream,
                               int64_t* pairs_kept);

/* Becke fuzzy-cell weights (host, FP64, OpenMP): for each point its
 * owner atom's cell weight.  Grid construction helper for the synthetic
 * workloads (PySCF builds the grids in the reference). */
int wb_becke_partition(const double* points, int64_t n, const int* owner,
                       const double* atom_coords, int natm, double* out);

/* FP32 FMA throughput probe: launches 8 CTAs per SM x 256 threads, each
 * thread 8 independent FMA chains for iters x 16 steps; *flops receives the
 * flop count of the launch (FMA = 2).  out needs nsm * 2048 floats.  The
 * caller times it (events on `stream`): the measured FP32 peak used as the
 * roofline denominator of the FP32-pipe kernels.  No reference counterpart
 * (the reference reports no roofline). */
int wb_fp32_fma_probe(int64_t iters, float* out, int64_t out_len,
                      void* stream, double* flops);
/* The same with packed FMAs (fma.rn.f32x2, two FP32 FMAs per instruction,
 * sm_100+): *flops counts both halves.  The FP32 peak of a roofline is the
 * larger of the two probes. */
int wb_fp32x2_fma_probe(int64_t iters, float* out, int64_t out_len, void* stream,
                        double* flops);

const char* wb_status_string(int status);
const char* wb_last_error(void);
int wb_version(void);

#ifdef __cplusplus
}
#endif
#endif /* WB97MV_GB300_H */
