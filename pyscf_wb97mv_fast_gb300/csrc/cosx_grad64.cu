// Integral-derivative part of the COSX exchange nuclear gradient (grid
// response off), in FP64:
//
//   E_w = -1/4 sum_g w_g sum_{nu,lam} F_g,nu A^g_nu,lam(w) F_g,lam,
//   F = X D.
//
// Moving a nucleus moves its basis functions.  The part of dE/dR that
// differentiates A is
//
//   -1/2 sum_g w_g sum_{nu on C} sum_lam F_g,nu F_g,lam d(nu lam|g)/dR_nu.
//
// It is collected per unordered shell pair (A, B): the bra derivative goes
// to atom(A) and the ket derivative to atom(B); a diagonal pair (B = A)
// contributes its bra derivative only.  For a primitive pair,
//   d/dA_x (a b|g) = 2 alpha (a + 1_x, b|g) - a_x (a - 1_x, b|g),
// and the ket derivative follows from translational invariance,
//   d/dB = -d/dA - d/dC, with d/dC_x R_tuv(P - C) = -R_t+1,u,v.
// The X side of the gradient (d F / dR through the AO values) is formed
// from G and the AO gradients by the host (cosx.CosxEngine.k_grad).
//
// The screen, pair tables, Boys function and McMurchie-Davidson recurrences
// are those of the plain FP64 kernels (cosx_fp64.cuh).  One warp owns one
// 32-point block; per task every lane forms its point's six derivative
// sums (atom A xyz, atom B xyz) times -w_g / 2.  The warp reduces them in a
// fixed order and lane 0 adds them to the block's row of gbuf (nblk, natm,
// 3), which no other warp touches.  The rows are summed in a fixed order
// afterwards, so the result is bitwise reproducible.  Loops are runtime
// loops (local-memory arrays): this kernel runs once per geometry, not per
// SCF cycle.
#include "cosx_fp64.cuh"
#include "cosx_grad64.hpp"

namespace wb {
namespace {

constexpr int kGradThreads = 128;

// E^{i,j}_t along one axis for i <= ia, j <= jb (t <= i + j), [i][j][t] with
// fixed strides (4 + 1) x 4 x 8
constexpr int kEi = 5, kEj = 4, kEt = 8;
__device__ __forceinline__ void hermite64(const int ia, const int jb, const double p,
                                          const double xpa, const double xpb,
                                          double* E) {
    const double h = 0.5 / p;
    auto at = [&](int i, int j, int t) -> double& { return E[(i * kEj + j) * kEt + t]; };
    for (int i = 0; i <= ia; ++i)
        for (int j = 0; j <= jb; ++j)
            for (int t = 0; t < kEt; ++t) at(i, j, t) = 0.0;
    at(0, 0, 0) = 1.0;
    for (int i = 1; i <= ia; ++i)
        for (int t = 0; t <= i; ++t) {
            double v = xpa * at(i - 1, 0, t);
            if (t > 0) v = fma(h, at(i - 1, 0, t - 1), v);
            if (t + 1 <= i - 1) v = fma((double)(t + 1), at(i - 1, 0, t + 1), v);
            at(i, 0, t) = v;
        }
    for (int j = 1; j <= jb; ++j)
        for (int i = 0; i <= ia; ++i)
            for (int t = 0; t <= i + j; ++t) {
                double v = xpb * at(i, j - 1, t);
                if (t > 0) v = fma(h, at(i, j - 1, t - 1), v);
                if (t + 1 <= i + j - 1) v = fma((double)(t + 1), at(i, j - 1, t + 1), v);
                at(i, j, t) = v;
            }
}

// R_tuv (t + u + v <= L) at PC = (x, y, z) from r0[n] = R_000^(n), levels
// L .. 0 in place; R[(t * 8 + u) * 8 + v]
__device__ __forceinline__ void fill_r_rt(const int L, const double* r0, const double x,
                                          const double y, const double z, double* R) {
    auto at = [&](int t, int u, int v) -> double& { return R[(t * 8 + u) * 8 + v]; };
    for (int i = 0; i < 512; ++i) R[i] = 0.0;
    for (int n = L; n >= 0; --n) {
        const int m = L - n;
        for (int u = 0; u < m; ++u)
            for (int v = 0; v < m - u; ++v)
                for (int t = m - u - v; t >= 1; --t)
                    at(t, u, v) = (t >= 2 ? (t - 1) * at(t - 2, u, v) : 0.0) +
                                  x * at(t - 1, u, v);
        for (int v = 0; v < m; ++v)
            for (int u = m - v; u >= 1; --u)
                at(0, u, v) = (u >= 2 ? (u - 1) * at(0, u - 2, v) : 0.0) +
                              y * at(0, u - 1, v);
        for (int v = m; v >= 1; --v)
            at(0, 0, v) = (v >= 2 ? (v - 1) * at(0, 0, v - 2) : 0.0) + z * at(0, 0, v - 1);
        at(0, 0, 0) = r0[n];
    }
}

// Boys F_0..F_L for runtime L (<= 7) from the FP64 table (as f64::boys64)
__device__ __forceinline__ void boys64_rt(const int L, const double T,
                                          const double* __restrict__ tab, double* F) {
    if (T < 36.0) {
        const int k = __double2int_rn(T * 4.0);
        const double x = 0.25 * k - T;
        const double* row = tab + k * kBoys64Cols + L;
        double s = row[11];
        for (int j = 11; j >= 1; --j) s = fma(s * x, 1.0 / j, row[j - 1]);
        F[L] = s;
        const double e = exp(-T);
        for (int n = L - 1; n >= 0; --n) F[n] = fma(2.0 * T, F[n + 1], e) / (2 * n + 1);
    } else {
        F[0] = 0.88622692545275801365 * rsqrt(T);
        const double e = exp(-T);
        const double h = 0.5 / T;
        for (int n = 0; n < L; ++n) F[n + 1] = ((2 * n + 1) * F[n] - e) * h;
    }
}

template<int LA, int LB>
__global__ void __launch_bounds__(kGradThreads)
cosx_grad64_kernel(const CosxGradArgs A, const int cls, const int pair_begin,
                   const int pair_end) {
    constexpr int L = LA + LB;
    constexpr int NCA = (LA + 1) * (LA + 2) / 2, NCB = (LB + 1) * (LB + 2) / 2;
    constexpr int NA = 2 * LA + 1, NB = 2 * LB + 1;
    __shared__ double stab[kBoys64Nodes * kBoys64Cols];
    for (int i = threadIdx.x; i < kBoys64Nodes * kBoys64Cols; i += blockDim.x)
        stab[i] = A.boys[i];
    __syncthreads();
    const int lane = threadIdx.x & 31;
    const long long ld = A.ld;
    const int pp_begin = A.pp_begin[cls];
    const float4* __restrict__ bnd = A.bnd + pp_begin;
    const float* __restrict__ bpref = A.bpref + pp_begin;
    const double om2 = A.omega * A.omega;
    int cxa[NCA], cya[NCA], cza[NCA], cxb[NCB], cyb[NCB], czb[NCB];
    for (int c = 0; c < NCA; ++c) {
        cxa[c] = f64::cx(LA, c); cya[c] = f64::cy(LA, c); cza[c] = LA - cxa[c] - cya[c];
    }
    for (int c = 0; c < NCB; ++c) {
        cxb[c] = f64::cx(LB, c); cyb[c] = f64::cy(LB, c); czb[c] = LB - cxb[c] - cyb[c];
    }
    for (;;) {
        int blk = 0;
        if (lane == 0) blk = atomicAdd(A.work + cls, 1);
        blk = __shfl_sync(0xffffffffu, blk, 0);
        if (blk >= A.nblk) break;
        const int g0 = blk * 32 + lane;
        const bool ok = g0 < A.npts;
        const int g = ok ? g0 : A.npts - 1;
        const double gx = A.coords[3LL * g], gy = A.coords[3LL * g + 1],
                     gz = A.coords[3LL * g + 2];
        const double wh = ok ? -0.5 * A.weights[g] : 0.0;
        const double* __restrict__ Fp = A.F + g;
        const float4 cr = A.blk_cr[blk];
        const float* __restrict__ ms = A.blk_msh + (long long)blk * A.nvshell;
        double* __restrict__ grow = A.gbuf + (long long)blk * A.natm * 3;
        for (int c0 = pair_begin; c0 < pair_end; c0 += 32) {
            const int k = c0 + lane;
            bool keep = k < pair_end;
            if (keep && A.tol > 0.0f) {
                const int2 sh = A.pshell[k];
                keep = screen_pair(A.tol, bnd, bpref, cr, A.khdr[k], A.ptau[k],
                                   fmaxf(ms[sh.x], ms[sh.y]));
            }
            unsigned mask = __ballot_sync(0xffffffffu, keep);
            while (mask) {
                const int kk = c0 + __ffs(mask) - 1;
                mask &= mask - 1;
                const int4 hdr = A.khdr[kk];
                const int2 sh = A.pshell[kk];
                const int ia0 = hdr.x & 0xffff, ib0 = hdr.y & 0xffff;
                const int pp0 = pp_begin + hdr.z, npp = hdr.w & 0xffff;
                const bool diag = (hdr.w >> 16) != 0;
                const double Ax = A.vs_xyz[3 * sh.x], Ay = A.vs_xyz[3 * sh.x + 1],
                             Az = A.vs_xyz[3 * sh.x + 2];
                const double Bx = A.vs_xyz[3 * sh.y], By = A.vs_xyz[3 * sh.y + 1],
                             Bz = A.vs_xyz[3 * sh.y + 2];
                double sa[NA], sb[NB], fa[NCA], fb[NCB];
                for (int m = 0; m < NA; ++m) sa[m] = Fp[(long long)(ia0 + m) * ld];
                for (int m = 0; m < NB; ++m) sb[m] = Fp[(long long)(ib0 + m) * ld];
                f64::to_cart<LA>(A.c2s, sa, fa);
                f64::to_cart<LB>(A.c2s, sb, fb);
                double gA[3] = {0.0, 0.0, 0.0}, gC[3] = {0.0, 0.0, 0.0};
                for (int q = pp0; q < pp0 + npp; ++q) {
                    const double p = A.p[q], pref = A.pref[q], al = A.alpha[q];
                    const double Px = A.P[3LL * q], Py = A.P[3LL * q + 1],
                                 Pz = A.P[3LL * q + 2];
                    const double X = Px - gx, Y = Py - gy, Z = Pz - gz;
                    double th = 1.0, sth = 1.0;
                    if (A.omega > 0.0) {
                        th = om2 / (om2 + p);
                        sth = sqrt(th);
                    }
                    const double pth = p * th;
                    const double T = pth * (X * X + Y * Y + Z * Z);
                    double Fb[L + 2], r0[L + 2];
                    boys64_rt(L + 1, T, stab, Fb);
                    double c = pref * sth;
                    for (int n = 0; n <= L + 1; ++n) {
                        r0[n] = c * Fb[n];
                        c *= -2.0 * pth;
                    }
                    double R[512];
                    fill_r_rt(L + 1, r0, X, Y, Z, R);
                    double Ex[kEi * kEj * kEt], Ey[kEi * kEj * kEt], Ez[kEi * kEj * kEt];
                    hermite64(LA + 1, LB, p, Px - Ax, Px - Bx, Ex);
                    hermite64(LA + 1, LB, p, Py - Ay, Py - By, Ey);
                    hermite64(LA + 1, LB, p, Pz - Az, Pz - Bz, Ez);
                    // Hermite sum of E_x[i][i'] E_y[j][j'] E_z[k][k'] R shifted
                    // by (dt, du, dv)
                    auto hsum = [&](int i, int ip, int j, int jp, int kz, int kp, int dt,
                                    int du, int dv) -> double {
                        double s = 0.0;
                        for (int t = 0; t <= i + ip; ++t) {
                            const double ex = Ex[(i * kEj + ip) * kEt + t];
                            double su = 0.0;
                            for (int u = 0; u <= j + jp; ++u) {
                                const double ey = Ey[(j * kEj + jp) * kEt + u];
                                double sv = 0.0;
                                for (int v = 0; v <= kz + kp; ++v)
                                    sv = fma(Ez[(kz * kEj + kp) * kEt + v],
                                             R[((t + dt) * 8 + u + du) * 8 + v + dv], sv);
                                su = fma(ey, sv, su);
                            }
                            s = fma(ex, su, s);
                        }
                        return s;
                    };
#pragma unroll 1
                    for (int a = 0; a < NCA; ++a) {
                        const int i = cxa[a], j = cya[a], kz = cza[a];
#pragma unroll 1
                        for (int b = 0; b < NCB; ++b) {
                            const int ip = cxb[b], jp = cyb[b], kp = czb[b];
                            const double ff = fa[a] * fb[b];
                            // bra derivative: 2 alpha (a + 1) - a_x (a - 1)
                            double dx = 2.0 * al * hsum(i + 1, ip, j, jp, kz, kp, 0, 0, 0);
                            if (i) dx -= i * hsum(i - 1, ip, j, jp, kz, kp, 0, 0, 0);
                            double dy = 2.0 * al * hsum(i, ip, j + 1, jp, kz, kp, 0, 0, 0);
                            if (j) dy -= j * hsum(i, ip, j - 1, jp, kz, kp, 0, 0, 0);
                            double dz = 2.0 * al * hsum(i, ip, j, jp, kz + 1, kp, 0, 0, 0);
                            if (kz) dz -= kz * hsum(i, ip, j, jp, kz - 1, kp, 0, 0, 0);
                            gA[0] = fma(ff, dx, gA[0]);
                            gA[1] = fma(ff, dy, gA[1]);
                            gA[2] = fma(ff, dz, gA[2]);
                            if (!diag) {
                                // operator-centre derivative: d/dC R_tuv = -R_t+1
                                gC[0] = fma(ff, -hsum(i, ip, j, jp, kz, kp, 1, 0, 0), gC[0]);
                                gC[1] = fma(ff, -hsum(i, ip, j, jp, kz, kp, 0, 1, 0), gC[1]);
                                gC[2] = fma(ff, -hsum(i, ip, j, jp, kz, kp, 0, 0, 1), gC[2]);
                            }
                        }
                    }
                }
                // atom(A): bra; atom(B): -(bra + operator centre)
                double v[6];
                for (int x = 0; x < 3; ++x) {
                    v[x] = wh * gA[x];
                    v[3 + x] = diag ? 0.0 : -wh * (gA[x] + gC[x]);
                }
                for (int x = 0; x < 6; ++x)
                    for (int o = 16; o > 0; o >>= 1)
                        v[x] += __shfl_xor_sync(0xffffffffu, v[x], o);
                if (lane == 0) {
                    const int atA = A.vs_atom[sh.x], atB = A.vs_atom[sh.y];
                    for (int x = 0; x < 3; ++x) grow[3 * atA + x] += v[x];
                    if (!diag)
                        for (int x = 0; x < 3; ++x) grow[3 * atB + x] += v[3 + x];
                }
                __syncwarp();
            }
        }
    }
}

template<int LA, int LB>
cudaError_t run_grad(const CosxGradArgs& a, int cls, int pb, int pe, int nsm,
                     cudaStream_t s) {
    const int warps = kGradThreads / 32;
    int grid = std::max(1, nsm * 4);
    grid = std::min(grid, (a.nblk + warps - 1) / warps);
    cosx_grad64_kernel<LA, LB><<<std::max(grid, 1), kGradThreads, 0, s>>>(a, cls, pb, pe);
    return cudaGetLastError();
}

__global__ void grad_rows_sum_kernel(const double* __restrict__ gbuf, int nblk, int n,
                                     double* __restrict__ out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double s = 0.0;
    for (int b = 0; b < nblk; ++b) s += gbuf[(long long)b * n + i];
    out[i] += s;
}

}  // namespace

cudaError_t launch_cosx_grad64_class(int cls, const CosxGradArgs& a, int pb, int pe,
                                     int nsm, cudaStream_t s) {
    switch (cls) {
    case 0: return run_grad<0, 0>(a, cls, pb, pe, nsm, s);
    case 1: return run_grad<1, 0>(a, cls, pb, pe, nsm, s);
    case 2: return run_grad<1, 1>(a, cls, pb, pe, nsm, s);
    case 3: return run_grad<2, 0>(a, cls, pb, pe, nsm, s);
    case 4: return run_grad<2, 1>(a, cls, pb, pe, nsm, s);
    case 5: return run_grad<2, 2>(a, cls, pb, pe, nsm, s);
    case 6: return run_grad<3, 0>(a, cls, pb, pe, nsm, s);
    case 7: return run_grad<3, 1>(a, cls, pb, pe, nsm, s);
    case 8: return run_grad<3, 2>(a, cls, pb, pe, nsm, s);
    case 9: return run_grad<3, 3>(a, cls, pb, pe, nsm, s);
    default: return cudaErrorInvalidValue;
    }
}

cudaError_t launch_grad_rows_sum(const double* gbuf, int nblk, int natm, double* out,
                                 cudaStream_t s) {
    const int n = 3 * natm;
    grad_rows_sum_kernel<<<(n + 127) / 128, 128, 0, s>>>(gbuf, nblk, n, out);
    return cudaGetLastError();
}

}  // namespace wb

namespace wb {
namespace {

__global__ void ao_dot_kernel(const double* __restrict__ dX, const double* __restrict__ H,
                              const double* __restrict__ w, int64_t npts, int64_t ld,
                              int nao, double* __restrict__ out) {
    __shared__ double red[3][256];
    const int mu = blockIdx.x;
    double s[3] = {0.0, 0.0, 0.0};
    const double* h = H + (int64_t)mu * ld;
    for (int64_t g = threadIdx.x; g < npts; g += blockDim.x) {
        const double wh = w[g] * h[g];
        for (int x = 0; x < 3; ++x)
            s[x] = fma(wh, dX[((int64_t)(1 + x) * nao + mu) * ld + g], s[x]);
    }
    for (int x = 0; x < 3; ++x) red[x][threadIdx.x] = s[x];
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
        if ((int)threadIdx.x < o)
            for (int x = 0; x < 3; ++x) red[x][threadIdx.x] += red[x][threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0)
        for (int x = 0; x < 3; ++x) out[3 * mu + x] = red[x][0];
}

__global__ void atom_sum_kernel(const double* __restrict__ aodot,
                                const int* __restrict__ vs_ao0,
                                const int* __restrict__ vs_nf,
                                const int* __restrict__ vs_atom, int nvshell, int natm,
                                double scale, double* __restrict__ grad) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= 3 * natm) return;
    const int at = i / 3, x = i % 3;
    double s = 0.0;
    for (int v = 0; v < nvshell; ++v)
        if (vs_atom[v] == at)
            for (int m = 0; m < vs_nf[v]; ++m) s += aodot[3 * (vs_ao0[v] + m) + x];
    grad[i] += scale * s;
}

}  // namespace

cudaError_t launch_ao_dot(const double* dX, const double* H, const double* w,
                          int64_t npts, int64_t ld, int nao, double* out,
                          cudaStream_t s) {
    ao_dot_kernel<<<nao, 256, 0, s>>>(dX, H, w, npts, ld, nao, out);
    return cudaGetLastError();
}

cudaError_t launch_atom_sum(const double* aodot, const int* vs_ao0, const int* vs_nf,
                            const int* vs_atom, int nvshell, int natm, double scale,
                            double* grad, cudaStream_t s) {
    const int n = 3 * natm;
    atom_sum_kernel<<<(n + 127) / 128, 128, 0, s>>>(aodot, vs_ao0, vs_nf, vs_atom,
                                                    nvshell, natm, scale, grad);
    return cudaGetLastError();
}

}  // namespace wb
