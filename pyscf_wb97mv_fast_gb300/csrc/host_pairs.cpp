// Host FP64 preprocessing of the COSX exchange: the shell-pair tables the
// fused G kernels read, the Boys table, Becke cell weights.
//
// Follows the data definitions of the reference's ShellPairs
// (pyscf_wb97mv_fast/gpu/shellpairs.py): pairs ish >= jsh kept by the
// primitive magnitude test sum_ab K_AB |c|max |c|max > cutoff (:248-297),
// per primitive pair p, P, K_AB 2 pi / p (:316-324), McMurchie-Davidson
// Hermite E^{i,i'}_t by the recurrence of _hermite_row (:76-113, :326-352)
// and the screening-bound data p' = 0.75 p, C_ab, pref, tau (:354-370,
// :123-168).  The layout is this library's own: pairs are oriented so
// that l_A >= l_B (10 kernel classes instead of 16), sorted by class, a
// generally contracted shell is split into one segmented "virtual" shell
// per contraction column (same AO columns), and the contraction
// coefficients, K_AB 2 pi / p and the s/p spherical normalisation are
// folded into one FP64 prefactor per primitive pair.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <numeric>

#include "host.hpp"
#include "generated/cosx_layout.h"

namespace wb {

void cart_components(int l, std::vector<int>& ix, std::vector<int>& iy,
                     std::vector<int>& iz) {
    ix.clear(); iy.clear(); iz.clear();
    for (int lx = l; lx >= 0; --lx)
        for (int ly = l - lx; ly >= 0; --ly) {
            ix.push_back(lx); iy.push_back(ly); iz.push_back(l - lx - ly);
        }
}

static double binom(int n, int k) {
    if (k < 0 || k > n) return 0.0;
    double r = 1.0;
    for (int i = 1; i <= k; ++i) r = r * (n - k + i) / i;
    return r;
}

static double fact(int n) {
    double r = 1.0;
    for (int i = 2; i <= n; ++i) r *= i;
    return r;
}

// real solid harmonic S_lm, Helgaker-Jorgensen-Olsen eq. 6.4.47-50, added
// into column `col` of the (ncart, nsph) matrix times `scale`
static void add_solid_harmonic(int l, int m, int col, double scale,
                               std::vector<double>& out) {
    std::vector<int> ix, iy, iz;
    cart_components(l, ix, iy, iz);
    const int nc = (int)ix.size(), ns = nsph(l);
    const int am = std::abs(m);
    const double vm = m >= 0 ? 0.0 : 0.5;
    const double nlm = (1.0 / (std::pow(2.0, am) * fact(l))) *
        std::sqrt(2.0 * fact(l + am) * fact(l - am) / (m == 0 ? 2.0 : 1.0));
    for (int t = 0; t <= (l - am) / 2; ++t)
        for (int u = 0; u <= t; ++u) {
            const double vmax = std::floor(am / 2.0 - vm) + vm;
            for (double v = vm; v <= vmax + 1e-12; v += 1.0) {
                const int two_v = (int)std::lround(2 * v);
                const int sgn = ((int)std::lround(t + v - vm)) % 2 ? -1 : 1;
                const double c = sgn * std::pow(0.25, t) * binom(l, t) *
                                 binom(l - t, am + t) * binom(t, u) *
                                 binom(am, two_v);
                const int ex = 2 * t + am - 2 * u - two_v;
                const int ey = 2 * u + two_v;
                const int ez = l - 2 * t - am;
                for (int k = 0; k < nc; ++k)
                    if (ix[k] == ex && iy[k] == ey && iz[k] == ez)
                        out[(size_t)k * ns + col] += nlm * c * scale;
            }
        }
}

std::vector<double> cart2sph(int l) {
    const int nc = ncart(l), ns = nsph(l);
    std::vector<double> out((size_t)nc * ns, 0.0);
    const double scale = std::sqrt((2 * l + 1) / (4.0 * M_PI));
    if (l == 1) {
        const int ms[3] = {1, -1, 0};
        for (int c = 0; c < 3; ++c) add_solid_harmonic(1, ms[c], c, scale, out);
    } else {
        for (int m = -l; m <= l; ++m)
            add_solid_harmonic(l, m, m + l, scale, out);
    }
    return out;
}

double c2s_tau(int l) {
    const std::vector<double> c = cart2sph(l);
    const int nc = ncart(l), ns = nsph(l);
    double best = 0.0;
    for (int s = 0; s < ns; ++s) {
        double acc = 0.0;
        for (int k = 0; k < nc; ++k) acc += std::fabs(c[(size_t)k * ns + s]);
        best = std::max(best, acc);
    }
    return best;
}

void boys_f64(int nmax, double t, double* out) {
    if (t < 40.0) {
        // F_nmax(t) = e^{-t} sum_i (2t)^i / ((2n+1)(2n+3)...(2n+2i+1))
        double term = 1.0 / (2 * nmax + 1), sum = term;
        for (int i = 1; i < 2000; ++i) {
            term *= 2.0 * t / (2 * nmax + 2 * i + 1);
            sum += term;
            if (term < 1e-18 * sum) break;
        }
        const double et = std::exp(-t);
        out[nmax] = et * sum;
        for (int n = nmax - 1; n >= 0; --n)
            out[n] = (2.0 * t * out[n + 1] + et) / (2 * n + 1);
    } else {
        const double et = std::exp(-t);
        out[0] = 0.5 * std::sqrt(M_PI / t) * std::erf(std::sqrt(t));
        for (int n = 0; n < nmax; ++n)
            out[n + 1] = ((2 * n + 1) * out[n] - et) / (2.0 * t);
    }
}

// Row layout per node (20 floats, float4 aligned): hi = fl32(F_m(T_k)),
// lo = fl32(F_m - hi):
//   [h0 h1 h2 h3 | h4 h5 h6 l0 | h7 l1 h8 l2 | h9 l3 h10 l4 | h11 l5 h12 l6]
// so an order-L evaluation (F_0..F_{L+6} hi, F_0..F_L lo) reads the first
// 2 + ceil(L / 2) float4s.
int boys_row_hi(int m) {
    if (m <= 6) return m;
    return 8 + 2 * (m - 7);
}
int boys_row_lo(int n) {
    if (n == 0) return 7;
    return 9 + 2 * (n - 1);
}

std::vector<float> boys_table() {
    std::vector<float> tab((size_t)BOYS_NODES * BOYS_ROW, 0.0f);
    double f[13];
    for (int k = 0; k < BOYS_NODES; ++k) {
        boys_f64(12, 0.25 * k, f);
        float* row = &tab[(size_t)k * BOYS_ROW];
        for (int m = 0; m <= 12; ++m) row[boys_row_hi(m)] = (float)f[m];
        for (int n = 0; n <= 6; ++n) {
            const float hi = (float)f[n];
            row[boys_row_lo(n)] = (float)(f[n] - (double)hi);
        }
    }
    return tab;
}

int e_count_axis(int la, int lb) {
    int n = 0;
    for (int i = 0; i <= la; ++i)
        for (int j = 0; j <= lb; ++j) n += i + j + 1;
    return n - 1;
}

int e_stride(int la, int lb) {
    const int n = 3 * e_count_axis(la, lb);
    return (n + 3) / 4 * 4;
}

// E^{i,j}_t for i <= la, j <= lb along one axis (FP64), [i][j][t] with
// t <= 6, via E^{i+1,j}_t = E^{i,j}_{t-1}/(2p) + X_PA E^{i,j}_t
// + (t+1) E^{i,j}_{t+1} and the same in j with X_PB.
static void hermite_axis(int la, int lb, double p, double xpa, double xpb,
                         double E[4][4][7]) {
    std::memset(E, 0, sizeof(double) * 4 * 4 * 7);
    const double inv2p = 0.5 / p;
    E[0][0][0] = 1.0;
    for (int i = 1; i <= la; ++i)
        for (int t = 0; t <= i; ++t) {
            double v = 0.0;
            if (t > 0) v += E[i - 1][0][t - 1] * inv2p;
            if (t <= i - 1) v += xpa * E[i - 1][0][t];
            if (t + 1 <= i - 1) v += (t + 1) * E[i - 1][0][t + 1];
            E[i][0][t] = v;
        }
    for (int j = 1; j <= lb; ++j)
        for (int i = 0; i <= la; ++i)
            for (int t = 0; t <= i + j; ++t) {
                double v = 0.0;
                if (t > 0) v += E[i][j - 1][t - 1] * inv2p;
                if (t <= i + j - 1) v += xpb * E[i][j - 1][t];
                if (t + 1 <= i + j - 1) v += (t + 1) * E[i][j - 1][t + 1];
                E[i][j][t] = v;
            }
}

// sup_{s >= 0} (s + a)^la (s + b)^lb exp(-eta p s^2): the log-derivative
// la/(s+a) + lb/(s+b) - 2 eta p s is strictly decreasing, so its root is
// the maximiser (bisection in FP64); times 1.01 like the reference's
// safety factor (shellpairs.py:167).
static double bound_c(int la, int lb, double p, double a, double b) {
    if (la == 0 && lb == 0) return 1.0;
    const double eta = 0.25;
    auto dlog = [&](double s) {
        double v = -2.0 * eta * p * s;
        if (la) v += la / std::max(s + a, 1e-300);
        if (lb) v += lb / std::max(s + b, 1e-300);
        return v;
    };
    double lo = 0.0, hi = std::sqrt((la + lb) / (2.0 * eta * p)) * 1.0001 + 1e-12;
    if (dlog(0.0) <= 0.0) hi = 0.0;
    for (int it = 0; it < 200 && hi > lo; ++it) {
        const double mid = 0.5 * (lo + hi);
        if (dlog(mid) > 0.0) lo = mid; else hi = mid;
    }
    const double s = 0.5 * (lo + hi);
    const double f = std::pow(s + a, la) * std::pow(s + b, lb) *
                     std::exp(-eta * p * s * s);
    return f * 1.01;
}

int e64_axis(int la, int lb) { return e_count_axis(la, lb) + 1; }

void build_pairs64(const HostPairs& hp, HostPairs64& out) {
    out = HostPairs64();
    int lofc[NCLASS][2];
    for (int x = 0; x <= LMAX; ++x)
        for (int y = 0; y <= x; ++y) {
            lofc[class_of(x, y)][0] = x;
            lofc[class_of(x, y)][1] = y;
        }
    int64_t base = 0;
    for (int c = 0; c < NCLASS; ++c) {
        out.e_base[c] = base;
        base += (int64_t)(hp.cls[c].pp_end - hp.cls[c].pp_begin) * 3 *
                e64_axis(lofc[c][0], lofc[c][1]);
    }
    out.P.resize(3 * (size_t)hp.npp);
    out.alpha.resize((size_t)hp.npp);
    out.E.resize((size_t)base);
    // primitive pairs follow the pair order, bra primitive outer (as in
    // build_pairs), so pair k's first one is hdr[4k + 2]
    for (int k = 0; k < hp.npairs; ++k) {
        const VShell& A = hp.vsh[hp.pshell[2 * k]];
        const VShell& B = hp.vsh[hp.pshell[2 * k + 1]];
        const int c = hp.pclass[k], la = A.l, lb = B.l, nax = e64_axis(la, lb);
        int pp = hp.hdr[4 * k + 2];
        for (int a = 0; a < A.nprim; ++a)
            for (int bb = 0; bb < B.nprim; ++bb, ++pp) {
                const double al = A.exps[a], be = B.exps[bb], p = al + be;
                out.alpha[(size_t)pp] = al;
                double* e = out.E.data() + out.e_base[c] +
                            (int64_t)(pp - hp.cls[c].pp_begin) * 3 * nax;
                for (int x = 0; x < 3; ++x) {
                    const double P = (al * A.A[x] + be * B.A[x]) / p;
                    out.P[3 * (size_t)pp + x] = P;
                    double E[4][4][7];
                    hermite_axis(la, lb, p, P - A.A[x], P - B.A[x], E);
                    int q = 0;
                    for (int i = 0; i <= la; ++i)
                        for (int j = 0; j <= lb; ++j)
                            for (int t = 0; t <= i + j; ++t) e[x * nax + q++] = E[i][j][t];
                }
            }
    }
}

int64_t model_flops(int la, int lb, int npi, int npj, bool diag) {
    const int L = la + lb;
    const int NA = nsph(la), NB = nsph(lb);
    const int NCA = ncart(la), NCB = ncart(lb);
    std::vector<int> ax, ay, az, bx, by, bz;
    cart_components(la, ax, ay, az);
    cart_components(lb, bx, by, bz);
    int64_t herm = 0;
    for (int ca = 0; ca < NCA; ++ca)
        for (int cb = 0; cb < NCB; ++cb) {
            const int nt = ax[ca] + bx[cb] + 1, nu = ay[ca] + by[cb] + 1,
                      nv = az[ca] + bz[cb] + 1;
            herm += (int64_t)nt * nu + 3LL * nt * nu * nv + 1;
        }
    const int64_t c4 = (int64_t)std::llround(binom(L + 4, 4));
    const int64_t fprim = 11 + 14LL * (L + 1) + 3LL * (c4 - (L + 1)) + herm +
                          2LL * NCA * NB * NCB;
    return (int64_t)npi * npj * fprim + (int64_t)npi * 2 * NA * NB * NCA +
           (diag ? 2LL : 4LL) * NA * NB;
}

static float round_up(double x) {
    float f = (float)x;
    if ((double)f < x) f = std::nextafter(f, INFINITY);
    return f;
}

int build_pairs(const wb_basis& b, const double origin[3], double cutoff,
                HostPairs& out, std::string& err) {
    out = HostPairs();
    if (b.nbas < 0 || b.natm < 0) { err = "negative sizes"; return WB_ERR_INVALID_ARGUMENT; }
    // -- virtual (segmented) shells ------------------------------------------
    int ao = 0;
    for (int s = 0; s < b.nbas; ++s) {
        const int l = b.shell_l[s], np = b.shell_nprim[s], nc = b.shell_nctr[s];
        if (l < 0 || l > LMAX) {
            err = "shell " + std::to_string(s) + " has l=" + std::to_string(l) +
                  "; the COSX kernels support l <= 3";
            return WB_ERR_UNSUPPORTED;
        }
        if (np < 1 || nc < 1 || np > PPR_MAX || nc * nsph(l) > NIA_MAX) {
            err = "shell " + std::to_string(s) + ": nprim=" + std::to_string(np) +
                  " nctr=" + std::to_string(nc) + " exceed the packed caps (16, 16)";
            return WB_ERR_UNSUPPORTED;
        }
        const int at = b.shell_atom[s];
        if (at < 0 || at >= b.natm) { err = "bad shell atom"; return WB_ERR_INVALID_ARGUMENT; }
        for (int ci = 0; ci < nc; ++ci) {
            VShell v;
            v.phys = s; v.ci = ci; v.atom = at; v.l = l; v.nprim = np;
            v.ao0 = ao + ci * nsph(l);
            for (int k = 0; k < 3; ++k) v.A[k] = b.atom_coords[at * 3 + k] - origin[k];
            v.cmax = 0.0;
            for (int a = 0; a < np; ++a) {
                v.exps.push_back(b.exps[b.shell_exp_off[s] + a]);
                const double c = b.coeffs[b.shell_coef_off[s] + a * nc + ci];
                v.coef.push_back(c);
                v.cmax = std::max(v.cmax, std::fabs(c));
            }
            out.vsh.push_back(v);
        }
        ao += nc * nsph(l);
    }
    if (ao > 65535) {
        err = "nao=" + std::to_string(ao) + " exceeds 65535 (16-bit packed rows)";
        return WB_ERR_UNSUPPORTED;
    }
    out.nao = ao;
    out.nbas_phys = b.nbas;
    out.nvshell = (int)out.vsh.size();
    // position of each virtual shell's first AO among the AOs of its l
    std::vector<int> lrow(out.vsh.size());
    for (size_t s = 0; s < out.vsh.size(); ++s) {
        const VShell& v = out.vsh[s];
        out.vs_ao0.push_back(v.ao0);
        out.vs_nf.push_back(nsph(v.l));
        lrow[s] = out.nlao[v.l];
        out.nlao[v.l] += nsph(v.l);
    }
    const double s_fold[LMAX + 1] = {cart2sph(0)[0], cart2sph(1)[0], 1.0, 1.0};
    double tau_l[LMAX + 1];
    for (int l = 0; l <= LMAX; ++l) tau_l[l] = c2s_tau(l);

    // -- candidate pairs (reference enumeration: i >= j) ---------------------
    struct Cand { int ish, jsh, A, B, cls; };
    std::vector<Cand> kept;
    const int nv = out.nvshell;
    for (int i = 0; i < nv; ++i)
        for (int j = 0; j <= i; ++j) {
            const VShell& vi = out.vsh[i];
            const VShell& vj = out.vsh[j];
            double d2 = 0.0;
            for (int k = 0; k < 3; ++k) d2 += (vi.A[k] - vj.A[k]) * (vi.A[k] - vj.A[k]);
            double mag = 0.0;
            for (int a = 0; a < vi.nprim; ++a)
                for (int bb = 0; bb < vj.nprim; ++bb) {
                    const double al = vi.exps[a], be = vj.exps[bb];
                    mag += std::exp(-al * be / (al + be) * d2);
                }
            mag *= vi.cmax * vj.cmax;
            if (!(mag > cutoff)) continue;
            Cand c;
            c.ish = i; c.jsh = j;
            if (vi.l >= vj.l) { c.A = i; c.B = j; } else { c.A = j; c.B = i; }
            c.cls = class_of(out.vsh[c.A].l, out.vsh[c.B].l);
            kept.push_back(c);
        }
    // class-major, then bra shell A, then ket B: consecutive tasks of a
    // class share A (the kernels keep F_A and G_A in registers per run)
    std::stable_sort(kept.begin(), kept.end(), [](const Cand& x, const Cand& y) {
        if (x.cls != y.cls) return x.cls < y.cls;
        if (x.A != y.A) return x.A < y.A;
        return x.B < y.B;
    });
    out.npairs = (int)kept.size();

    // -- per pair / per primitive pair ---------------------------------------
    int pp = 0;
    int64_t ebase = 0;
    int cur_cls = -1;
    for (int c = 0; c < NCLASS; ++c) out.cls[c] = ClassRange();
    for (int k = 0; k < out.npairs; ++k) {
        const Cand& c = kept[k];
        const VShell& A = out.vsh[c.A];
        const VShell& B = out.vsh[c.B];
        const int la = A.l, lb = B.l, L = la + lb;
        if (c.cls != cur_cls) {
            // close the previous class, open this one
            if (cur_cls >= 0) {
                out.cls[cur_cls].pair_end = k;
                out.cls[cur_cls].pp_end = pp;
                const int cl = cur_cls;
                int lla = 0, llb = 0;
                for (int x = 0; x <= LMAX; ++x)
                    for (int y = 0; y <= x; ++y)
                        if (class_of(x, y) == cl) { lla = x; llb = y; }
                ebase += (int64_t)(out.cls[cl].pp_end - out.cls[cl].pp_begin) *
                         e_stride(lla, llb);
            }
            cur_cls = c.cls;
            out.cls[cur_cls].pair_begin = k;
            out.cls[cur_cls].pp_begin = pp;
            out.cls[cur_cls].e_base = ebase;
        }
        const bool diag = (c.A == c.B);
        const int npp = A.nprim * B.nprim;
        out.hdr.push_back(A.ao0);
        out.hdr.push_back(B.ao0);
        out.hdr.push_back(pp);
        out.hdr.push_back(npp | (diag ? (1 << 16) : 0));
        {
            const int ga0 = lrow[c.A];
            const int gb0 = (la != lb ? out.nlao[la] : 0) + lrow[c.B];
            out.khdr.push_back((int32_t)((uint32_t)A.ao0 | ((uint32_t)ga0 << 16)));
            out.khdr.push_back((int32_t)((uint32_t)B.ao0 | ((uint32_t)gb0 << 16)));
            out.khdr.push_back(pp - out.cls[c.cls].pp_begin);    // class-local
            out.khdr.push_back(npp | (diag ? (1 << 16) : 0));
        }
        out.pshell.push_back(c.A);
        out.pshell.push_back(c.B);
        out.pclass.push_back(c.cls);
        out.pish.push_back(c.ish);
        out.pjsh.push_back(c.jsh);
        {   // flop model in the reference orientation (bra = ish)
            const VShell& I = out.vsh[c.ish];
            const VShell& J = out.vsh[c.jsh];
            out.pflops.push_back(model_flops(I.l, J.l, I.nprim, J.nprim, diag));
        }
        out.pnint.push_back(nsph(la) * nsph(lb));

        double d2 = 0.0;
        for (int x = 0; x < 3; ++x) d2 += (A.A[x] - B.A[x]) * (A.A[x] - B.A[x]);
        const int nea = 3 * e_count_axis(la, lb), est = e_stride(la, lb);
        double prefsum = 0.0;
        for (int a = 0; a < A.nprim; ++a)
            for (int bb = 0; bb < B.nprim; ++bb) {
                const double al = A.exps[a], be = B.exps[bb];
                const double p = al + be, mu = al * be / p;
                double P[3];
                for (int x = 0; x < 3; ++x) P[x] = (al * A.A[x] + be * B.A[x]) / p;
                const double K = std::exp(-mu * d2);
                out.p.push_back(p);
                out.pref.push_back(A.coef[a] * B.coef[bb] * K * (2.0 * M_PI / p) *
                                   s_fold[la] * s_fold[lb]);
                for (int x = 0; x < 3; ++x) {
                    const float hi = (float)P[x];
                    out.geo.push_back(hi);
                }
                out.geo.push_back(0.0f);
                for (int x = 0; x < 3; ++x) {
                    const float hi = (float)P[x];
                    out.geo.push_back((float)(P[x] - (double)hi));
                }
                out.geo.push_back(0.0f);
                // Hermite coefficients, packed [axis][i][i'][t] minus E^{00}_0
                for (int x = 0; x < 3; ++x) {
                    double E[4][4][7];
                    hermite_axis(la, lb, p, P[x] - A.A[x], P[x] - B.A[x], E);
                    for (int i = 0; i <= la; ++i)
                        for (int j = 0; j <= lb; ++j)
                            for (int t = 0; t <= i + j; ++t) {
                                if (i == 0 && j == 0) continue;
                                out.E.push_back((float)E[i][j][t]);
                            }
                }
                for (int q = nea; q < est; ++q) out.E.push_back(0.0f);
                // screening bound (locked definition of the reference)
                double rpa = 0.0, rpb = 0.0;
                for (int x = 0; x < 3; ++x) {
                    rpa += (P[x] - A.A[x]) * (P[x] - A.A[x]);
                    rpb += (P[x] - B.A[x]) * (P[x] - B.A[x]);
                }
                const double cab = bound_c(la, lb, p, std::sqrt(rpa), std::sqrt(rpb));
                const double ppr = 0.75 * p;
                const double bp = std::fabs(A.coef[a]) * std::fabs(B.coef[bb]) * K *
                                  cab * (2.0 * M_PI / ppr);
                const float bpf = round_up(bp);
                out.bpref.push_back(bpf);
                prefsum += (double)bpf;
                for (int x = 0; x < 3; ++x) out.bnd.push_back((float)P[x]);
                out.bnd.push_back((float)ppr);
                ++pp;
            }
        const float tau = round_up(tau_l[la] * tau_l[lb]);
        out.ptau.push_back(tau);
        out.ptau.push_back(round_up((double)tau * round_up(prefsum)));
    }
    if (cur_cls >= 0) {
        out.cls[cur_cls].pair_end = out.npairs;
        out.cls[cur_cls].pp_end = pp;
    }
    // empty classes: zero-length ranges at the end of the previous one
    for (int c = 0; c < NCLASS; ++c)
        if (out.cls[c].pair_end == 0 && out.cls[c].pair_begin == 0 &&
            out.cls[c].pp_end == 0) {
            out.cls[c].pair_begin = out.cls[c].pair_end = 0;
            out.cls[c].pp_begin = out.cls[c].pp_end = 0;
        }
    out.npp = pp;
    // class partial-G buffers and the rows each AO of G sums
    int64_t base = 0;
    for (int la = 0; la <= LMAX; ++la)
        for (int lb = 0; lb <= la; ++lb) {
            const int c = class_of(la, lb);
            const bool used = out.cls[c].pair_end > out.cls[c].pair_begin;
            out.crow[c] = used ? out.nlao[la] + (la != lb ? out.nlao[lb] : 0) : 0;
            out.crow_base[c] = base;
            base += out.crow[c];
        }
    out.ncrow = base;
    // packed primitive-pair records (float4 offsets per class)
    for (int la = 0; la <= LMAX; ++la)
        for (int lb = 0; lb <= la; ++lb) {
            const int c = class_of(la, lb);
            if (kRecNe[c] * 4 != e_stride(la, lb) || kRecNom[c] != 2 + (la + lb + 1) / 2 ||
                kRecStride[c] != 2 + kRecNom[c] + kRecNe[c] ||
                kRecStride2[c] != 2 + 2 * kRecNom[c] + kRecNe[c]) {
                err = "generated record layout does not match the pair tables";
                return WB_ERR_UNSUPPORTED;
            }
        }
    int64_t roff = 0, roff2 = 0;
    for (int c = 0; c < NCLASS; ++c) {
        out.rec_off[c] = roff;
        out.rec_off2[c] = roff2;
        const int64_t n = out.cls[c].pp_end - out.cls[c].pp_begin;
        roff += n * kRecStride[c];
        roff2 += n * kRecStride2[c];
    }
    out.nrec = roff;
    out.nrec2 = roff2;
    out.gsrc.assign(4 * (size_t)out.nao, -1);
    for (size_t s = 0; s < out.vsh.size(); ++s) {
        const VShell& v = out.vsh[s];
        for (int comp = 0; comp < nsph(v.l); ++comp) {
            int n = 0;
            for (int c = 0; c < NCLASS; ++c) {
                if (!out.crow[c]) continue;
                int la = 0, lb = 0;
                for (int x = 0; x <= LMAX; ++x)
                    for (int y = 0; y <= x; ++y)
                        if (class_of(x, y) == c) { la = x; lb = y; }
                int64_t row = -1;
                if (la == v.l) row = out.crow_base[c] + lrow[s] + comp;
                else if (lb == v.l) row = out.crow_base[c] + out.nlao[la] + lrow[s] + comp;
                if (row < 0) continue;
                if (row > INT32_MAX) {
                    err = "partial-G rows exceed 2^31";
                    return WB_ERR_UNSUPPORTED;
                }
                out.gsrc[4 * (size_t)(v.ao0 + comp) + n++] = (int32_t)row;
            }
        }
    }
    return WB_OK;
}

void becke_partition(const double* pts, int64_t n, const int* owner,
                     const double* atoms, int natm, double* out) {
    std::vector<double> rinv((size_t)natm * natm, 0.0);
    for (int a = 0; a < natm; ++a)
        for (int b = 0; b < natm; ++b) {
            if (a == b) continue;
            double d2 = 0.0;
            for (int x = 0; x < 3; ++x) {
                const double d = atoms[a * 3 + x] - atoms[b * 3 + x];
                d2 += d * d;
            }
            rinv[(size_t)a * natm + b] = 1.0 / std::sqrt(d2);
        }
#pragma omp parallel
    {
        std::vector<double> dist(natm), P(natm);
#pragma omp for schedule(static)
        for (int64_t i = 0; i < n; ++i) {
            for (int a = 0; a < natm; ++a) {
                double d2 = 0.0;
                for (int x = 0; x < 3; ++x) {
                    const double d = pts[i * 3 + x] - atoms[a * 3 + x];
                    d2 += d * d;
                }
                dist[a] = std::sqrt(d2);
                P[a] = 1.0;
            }
            for (int a = 0; a < natm; ++a)
                for (int b = a + 1; b < natm; ++b) {
                    double mu = (dist[a] - dist[b]) * rinv[(size_t)a * natm + b];
                    for (int it = 0; it < 3; ++it) mu = 1.5 * mu - 0.5 * mu * mu * mu;
                    P[a] *= 0.5 * (1.0 - mu);
                    P[b] *= 0.5 * (1.0 + mu);
                }
            double tot = 0.0;
            for (int a = 0; a < natm; ++a) tot += P[a];
            out[i] = tot > 0.0 ? P[owner[i]] / tot : 0.0;
        }
    }
}

}  // namespace wb
