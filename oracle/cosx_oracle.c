/*
 * cosx_oracle.c -- FP64 CPU restatement of the reference's COSX math.
 *
 * TEST INFRASTRUCTURE ONLY: this is the checker of the GPU path (tests,
 * __graft_entry__.smoke, the cpu_baseline leg of bench.py).  Nothing in the
 * product library links, loads or calls it.
 *
 * Restates, in plain C with OpenMP over grid points:
 *   oracle_boys         F_n(T) in FP64 (the quantity of gpu/boys.py:66-77,
 *                       boys_ref; series + downward recursion, erf + upward
 *                       recursion for T >= 40)
 *   oracle_int3c1e      dense (mu|1/|r-g||nu) or erf(w r)/r, spherical,
 *                       contracted: gpu/shellpairs.py:499-542
 *                       (int3c1e_reference) with the Hermite recurrence of
 *                       :76-113 and the R recurrence of :447-485
 *   oracle_cosx_g       G_gv = sum_mu A^g_mu,v F_g,mu (+ transposed term for
 *                       ish != jsh): the contraction of gpu/sgx_k.py:127-148
 *   oracle_ao_eval      AO values, gpu/ao_eval.py:255-329 (deriv 0)
 *   oracle_vv10_sum     brute-force F, U, W of tests/gpu/test_xc_vv10.py:
 *                       257-266 (F = -1.5 x raw sum)
 * Inputs are the packed basis arrays of Molecule.packed() plus the
 * Cartesian -> spherical matrices (ncart, nsph) row-major for l = 0..3.
 * Pairs are enumerated as in the reference (ish >= jsh, all primitive
 * pairs); oracle_cosx_g applies the reference's shell-pair magnitude cut
 * (gpu/shellpairs.py:287-294) when given a cutoff > 0.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#define LMAX 3
#define ET (2 * LMAX + 1)

typedef struct {
    int natm, nbas;
    const double* atom_coords;
    const int *shell_atom, *shell_l, *shell_nprim, *shell_nctr;
    const int *shell_exp_off, *shell_coef_off;
    const double *exps, *coeffs;
    const double* c2s[4];
} obasis;

static int ncart(int l) { return (l + 1) * (l + 2) / 2; }
static int nsph(int l) { return 2 * l + 1; }

static void cart_comp(int l, int c, int* i, int* j, int* k) {
    int n = 0;
    for (int lx = l; lx >= 0; --lx)
        for (int ly = l - lx; ly >= 0; --ly) {
            if (n == c) { *i = lx; *j = ly; *k = l - lx - ly; return; }
            ++n;
        }
}

int oracle_boys(int nmax, double t, double* out) {
    if (nmax < 0 || t < 0.0) return 1;
    if (t < 40.0) {
        double term = 1.0 / (2 * nmax + 1), sum = term;
        for (int i = 1; i < 4000; ++i) {
            term *= 2.0 * t / (2 * nmax + 2 * i + 1);
            sum += term;
            if (term < 1e-18 * sum) break;
        }
        const double et = exp(-t);
        out[nmax] = et * sum;
        for (int n = nmax - 1; n >= 0; --n)
            out[n] = (2.0 * t * out[n + 1] + et) / (2 * n + 1);
    } else {
        const double et = exp(-t);
        out[0] = 0.5 * sqrt(M_PI / t) * erf(sqrt(t));
        for (int n = 0; n < nmax; ++n)
            out[n + 1] = ((2 * n + 1) * out[n] - et) / (2.0 * t);
    }
    return 0;
}

/* E^{i,j}_t along one axis, [i][j][t] */
static void hermite(int la, int lb, double p, double xpa, double xpb,
                    double E[LMAX + 1][LMAX + 1][ET]) {
    memset(E, 0, sizeof(double) * (LMAX + 1) * (LMAX + 1) * ET);
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

/* R_tuv (t+u+v <= L) at P - C = (x, y, z): levels L .. 0 in place */
static void fill_r(int L, double T, double pth, double sth, double x, double y,
                   double z, double R[ET][ET][ET]) {
    double F[ET];
    oracle_boys(L, T, F);
    double r000[ET];
    double q = -2.0 * pth, c = sth;
    for (int n = 0; n <= L; ++n) { r000[n] = c * F[n]; c *= q; }
    memset(R, 0, sizeof(double) * ET * ET * ET);
    for (int n = L; n >= 0; --n) {
        const int m = L - n;
        for (int u = 0; u < m; ++u)
            for (int v = 0; v < m - u; ++v)
                for (int t = m - u - v; t >= 1; --t)
                    R[t][u][v] = (t == 1) ? x * R[0][u][v]
                                          : (t - 1) * R[t - 2][u][v] + x * R[t - 1][u][v];
        for (int v = 0; v < m; ++v)
            for (int u = m - v; u >= 1; --u)
                R[0][u][v] = (u == 1) ? y * R[0][0][v]
                                      : (u - 1) * R[0][u - 2][v] + y * R[0][u - 1][v];
        for (int v = m; v >= 1; --v)
            R[0][0][v] = (v == 1) ? z * R[0][0][0]
                                  : (v - 1) * R[0][0][v - 2] + z * R[0][0][v - 1];
        R[0][0][0] = r000[n];
    }
}

/* contracted spherical block A[(ci, mu), (cj, nu)] of shells (ish, jsh) at
 * point g; returns ni, nj through the pointers; A has row stride 16 */
static void pair_block(const obasis* b, int ish, int jsh, const double* g,
                       double omega, double* A, int* pni, int* pnj) {
    const int la = b->shell_l[ish], lb = b->shell_l[jsh], L = la + lb;
    const int npi = b->shell_nprim[ish], npj = b->shell_nprim[jsh];
    const int nci = b->shell_nctr[ish], ncj = b->shell_nctr[jsh];
    const int nca = ncart(la), ncb = ncart(lb), nsa = nsph(la), nsb = nsph(lb);
    const double* Ac_ = b->atom_coords + 3 * b->shell_atom[ish];
    const double* Bc_ = b->atom_coords + 3 * b->shell_atom[jsh];
    const double* ea = b->exps + b->shell_exp_off[ish];
    const double* eb = b->exps + b->shell_exp_off[jsh];
    const double* ca = b->coeffs + b->shell_coef_off[ish];
    const double* cb = b->coeffs + b->shell_coef_off[jsh];
    const int ni = nci * nsa, nj = ncj * nsb;
    *pni = ni; *pnj = nj;
    double cart[10 * 10];
    double R[ET][ET][ET];
    double Ex[LMAX + 1][LMAX + 1][ET], Ey[LMAX + 1][LMAX + 1][ET],
        Ez[LMAX + 1][LMAX + 1][ET];
    for (int i = 0; i < 16 * 16; ++i) A[i] = 0.0;
    double d2 = 0.0;
    for (int x = 0; x < 3; ++x) d2 += (Ac_[x] - Bc_[x]) * (Ac_[x] - Bc_[x]);
    for (int a = 0; a < npi; ++a)
        for (int bb = 0; bb < npj; ++bb) {
            const double al = ea[a], be = eb[bb], p = al + be, mu = al * be / p;
            double P[3];
            for (int x = 0; x < 3; ++x) P[x] = (al * Ac_[x] + be * Bc_[x]) / p;
            const double K = exp(-mu * d2);
            double th = 1.0, sth = 1.0;
            if (omega > 0.0) {
                th = omega * omega / (omega * omega + p);
                sth = sqrt(th);
            }
            const double px = P[0] - g[0], py = P[1] - g[1], pz = P[2] - g[2];
            const double r2 = px * px + py * py + pz * pz;
            fill_r(L, th * p * r2, p * th, sth, px, py, pz, R);
            hermite(la, lb, p, P[0] - Ac_[0], P[0] - Bc_[0], Ex);
            hermite(la, lb, p, P[1] - Ac_[1], P[1] - Bc_[1], Ey);
            hermite(la, lb, p, P[2] - Ac_[2], P[2] - Bc_[2], Ez);
            const double pf = K * 2.0 * M_PI / p;
            for (int qa = 0; qa < nca; ++qa) {
                int i, j, k;
                cart_comp(la, qa, &i, &j, &k);
                for (int qb = 0; qb < ncb; ++qb) {
                    int ip, jp, kp;
                    cart_comp(lb, qb, &ip, &jp, &kp);
                    double s = 0.0;
                    for (int t = 0; t <= i + ip; ++t)
                        for (int u = 0; u <= j + jp; ++u)
                            for (int v = 0; v <= k + kp; ++v)
                                s += Ex[i][ip][t] * Ey[j][jp][u] * Ez[k][kp][v] * R[t][u][v];
                    cart[qa * ncb + qb] = pf * s;
                }
            }
            /* contract: A[(ci,mu),(cj,nu)] += C_a,ci C_b,cj c2s_a[qa,mu]
             * cart[qa,qb] c2s_b[qb,nu] */
            for (int ci = 0; ci < nci; ++ci)
                for (int cj = 0; cj < ncj; ++cj) {
                    const double cc = ca[a * nci + ci] * cb[bb * ncj + cj];
                    for (int m1 = 0; m1 < nsa; ++m1)
                        for (int m2 = 0; m2 < nsb; ++m2) {
                            double s = 0.0;
                            for (int qa = 0; qa < nca; ++qa) {
                                const double c1 = b->c2s[la][qa * nsa + m1];
                                if (c1 == 0.0) continue;
                                for (int qb = 0; qb < ncb; ++qb)
                                    s += c1 * cart[qa * ncb + qb] * b->c2s[lb][qb * nsb + m2];
                            }
                            A[(ci * nsa + m1) * 16 + cj * nsb + m2] += cc * s;
                        }
                }
        }
}

static void make_basis(obasis* b, int natm, int nbas, const double* atom_coords,
                       const int* shell_atom, const int* shell_l,
                       const int* shell_nprim, const int* shell_nctr,
                       const int* shell_exp_off, const int* shell_coef_off,
                       const double* exps, const double* coeffs,
                       const double* c2s0, const double* c2s1,
                       const double* c2s2, const double* c2s3) {
    b->natm = natm; b->nbas = nbas; b->atom_coords = atom_coords;
    b->shell_atom = shell_atom; b->shell_l = shell_l;
    b->shell_nprim = shell_nprim; b->shell_nctr = shell_nctr;
    b->shell_exp_off = shell_exp_off; b->shell_coef_off = shell_coef_off;
    b->exps = exps; b->coeffs = coeffs;
    b->c2s[0] = c2s0; b->c2s[1] = c2s1; b->c2s[2] = c2s2; b->c2s[3] = c2s3;
}

static int* ao_offsets(const obasis* b) {
    int* ao = (int*)malloc(sizeof(int) * (b->nbas + 1));
    ao[0] = 0;
    for (int s = 0; s < b->nbas; ++s)
        ao[s + 1] = ao[s] + b->shell_nctr[s] * nsph(b->shell_l[s]);
    return ao;
}

#define OBASIS_ARGS                                                         \
    int natm, int nbas, const double *atom_coords, const int *shell_atom,   \
        const int *shell_l, const int *shell_nprim, const int *shell_nctr,  \
        const int *shell_exp_off, const int *shell_coef_off,                \
        const double *exps, const double *coeffs, const double *c2s0,       \
        const double *c2s1, const double *c2s2, const double *c2s3
#define OBASIS_PASS                                                         \
    natm, nbas, atom_coords, shell_atom, shell_l, shell_nprim, shell_nctr,  \
        shell_exp_off, shell_coef_off, exps, coeffs, c2s0, c2s1, c2s2, c2s3

/* out (ng, nao, nao) */
int oracle_int3c1e(OBASIS_ARGS, const double* coords, int64_t ng, double omega,
                   double* out) {
    obasis b;
    make_basis(&b, OBASIS_PASS);
    int* ao = ao_offsets(&b);
    const int nao = ao[nbas];
#pragma omp parallel for schedule(dynamic, 1)
    for (int64_t g = 0; g < ng; ++g) {
        double A[256];
        double* row = out + g * (int64_t)nao * nao;
        for (int ish = 0; ish < nbas; ++ish)
            for (int jsh = 0; jsh <= ish; ++jsh) {
                int ni, nj;
                pair_block(&b, ish, jsh, coords + 3 * g, omega, A, &ni, &nj);
                for (int m1 = 0; m1 < ni; ++m1)
                    for (int m2 = 0; m2 < nj; ++m2) {
                        const double v = A[m1 * 16 + m2];
                        row[(int64_t)(ao[ish] + m1) * nao + ao[jsh] + m2] = v;
                        row[(int64_t)(ao[jsh] + m2) * nao + ao[ish] + m1] = v;
                    }
            }
    }
    free(ao);
    return 0;
}

/* The reference's shell-pair cut (gpu/shellpairs.py:287-294): a pair
 * (ish >= jsh) is kept when sum_ab exp(-a b / (a + b) |A - B|^2) times the
 * two shells' largest |contraction coefficient| exceeds cutoff (0 keeps
 * every pair).  keep (nbas, nbas), lower triangle used. */
static unsigned char* pair_keep(const obasis* b, double cutoff) {
    const int n = b->nbas;
    unsigned char* keep = (unsigned char*)malloc((size_t)n * n);
    double* cmax = (double*)calloc((size_t)n, sizeof(double));
    for (int s = 0; s < n; ++s) {
        const int np = b->shell_nprim[s], nc = b->shell_nctr[s];
        for (int k = 0; k < np * nc; ++k)
            cmax[s] = fmax(cmax[s], fabs(b->coeffs[b->shell_coef_off[s] + k]));
    }
    for (int i = 0; i < n; ++i)
        for (int j = 0; j <= i; ++j) {
            const double* A = b->atom_coords + 3 * b->shell_atom[i];
            const double* B = b->atom_coords + 3 * b->shell_atom[j];
            const double d2 = (A[0] - B[0]) * (A[0] - B[0]) +
                              (A[1] - B[1]) * (A[1] - B[1]) +
                              (A[2] - B[2]) * (A[2] - B[2]);
            double mag = 0.0;
            for (int a = 0; a < b->shell_nprim[i]; ++a)
                for (int c = 0; c < b->shell_nprim[j]; ++c) {
                    const double al = b->exps[b->shell_exp_off[i] + a];
                    const double be = b->exps[b->shell_exp_off[j] + c];
                    mag += exp(-al * be / (al + be) * d2);
                }
            keep[(size_t)i * n + j] = cutoff <= 0.0 || mag * cmax[i] * cmax[j] > cutoff;
        }
    free(cmax);
    return keep;
}

/* The pair cut alone, for the work credit of the CPU baselines: keep
 * (nbas, nbas), 1 where pair (i >= j) is kept, lower triangle filled. */
int oracle_pair_keep(OBASIS_ARGS, double cutoff, unsigned char* keep) {
    obasis b;
    make_basis(&b, OBASIS_PASS);
    unsigned char* k = pair_keep(&b, cutoff);
    if (!k) return 1;
    for (size_t i = 0; i < (size_t)nbas * nbas; ++i) keep[i] = 0;
    for (int i = 0; i < nbas; ++i)
        for (int j = 0; j <= i; ++j) keep[(size_t)i * nbas + j] = k[(size_t)i * nbas + j];
    free(k);
    return 0;
}

/* F, G (ng, nao) point-major; G overwritten.  Only the shell pairs that
 * pair_keep keeps contribute. */
int oracle_cosx_g(OBASIS_ARGS, const double* coords, int64_t ng, double omega,
                  double cutoff, const double* F, double* G) {
    obasis b;
    make_basis(&b, OBASIS_PASS);
    int* ao = ao_offsets(&b);
    const int nao = ao[nbas];
    unsigned char* keep = pair_keep(&b, cutoff);
#pragma omp parallel for schedule(dynamic, 1)
    for (int64_t g = 0; g < ng; ++g) {
        double A[256];
        const double* Fg = F + g * (int64_t)nao;
        double* Gg = G + g * (int64_t)nao;
        for (int i = 0; i < nao; ++i) Gg[i] = 0.0;
        for (int ish = 0; ish < nbas; ++ish)
            for (int jsh = 0; jsh <= ish; ++jsh) {
                if (!keep[(size_t)ish * nbas + jsh]) continue;
                int ni, nj;
                pair_block(&b, ish, jsh, coords + 3 * g, omega, A, &ni, &nj);
                const int i0 = ao[ish], j0 = ao[jsh];
                for (int nu = 0; nu < nj; ++nu) {
                    double s = 0.0;
                    for (int mu = 0; mu < ni; ++mu) s += A[mu * 16 + nu] * Fg[i0 + mu];
                    Gg[j0 + nu] += s;
                }
                if (ish != jsh)
                    for (int mu = 0; mu < ni; ++mu) {
                        double s = 0.0;
                        for (int nu = 0; nu < nj; ++nu) s += A[mu * 16 + nu] * Fg[j0 + nu];
                        Gg[i0 + mu] += s;
                    }
            }
    }
    free(keep);
    free(ao);
    return 0;
}

/* X (ng, nao) point-major */
int oracle_ao_eval(OBASIS_ARGS, const double* coords, int64_t ng, double* X) {
    obasis b;
    make_basis(&b, OBASIS_PASS);
    int* ao = ao_offsets(&b);
    const int nao = ao[nbas];
#pragma omp parallel for schedule(static)
    for (int64_t g = 0; g < ng; ++g) {
        for (int s = 0; s < nbas; ++s) {
            const int l = shell_l[s], np = shell_nprim[s], nc = shell_nctr[s];
            const double* A = atom_coords + 3 * shell_atom[s];
            const double dx = coords[3 * g] - A[0], dy = coords[3 * g + 1] - A[1],
                         dz = coords[3 * g + 2] - A[2];
            const double r2 = dx * dx + dy * dy + dz * dz;
            const int nca = ncart(l), ns = nsph(l);
            double mono[10];
            for (int c = 0; c < nca; ++c) {
                int i, j, k;
                cart_comp(l, c, &i, &j, &k);
                mono[c] = pow(dx, i) * pow(dy, j) * pow(dz, k);
            }
            for (int ci = 0; ci < nc; ++ci) {
                double rad = 0.0;
                for (int k = 0; k < np; ++k)
                    rad += coeffs[shell_coef_off[s] + k * nc + ci] *
                           exp(-exps[shell_exp_off[s] + k] * r2);
                for (int m = 0; m < ns; ++m) {
                    double v = 0.0;
                    for (int c = 0; c < nca; ++c) v += b.c2s[l][c * ns + m] * mono[c];
                    X[g * (int64_t)nao + ao[s] + ci * ns + m] = rad * v;
                }
            }
        }
    }
    free(ao);
    return 0;
}

/* X (4, ng, nao): values and x, y, z gradients */
int oracle_ao_eval_deriv1(OBASIS_ARGS, const double* coords, int64_t ng,
                          double* X) {
    obasis b;
    make_basis(&b, OBASIS_PASS);
    int* ao = ao_offsets(&b);
    const int nao = ao[nbas];
    const int64_t plane = ng * (int64_t)nao;
#pragma omp parallel for schedule(static)
    for (int64_t g = 0; g < ng; ++g) {
        for (int s = 0; s < nbas; ++s) {
            const int l = shell_l[s], np = shell_nprim[s], nc = shell_nctr[s];
            const double* A = atom_coords + 3 * shell_atom[s];
            const double d[3] = {coords[3 * g] - A[0], coords[3 * g + 1] - A[1],
                                 coords[3 * g + 2] - A[2]};
            const double r2 = d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
            const int nca = ncart(l), ns = nsph(l);
            for (int ci = 0; ci < nc; ++ci) {
                double cart[4][10];
                for (int c = 0; c < nca; ++c) {
                    int e[3];
                    cart_comp(l, c, &e[0], &e[1], &e[2]);
                    double val = 0.0, gr[3] = {0.0, 0.0, 0.0};
                    for (int k = 0; k < np; ++k) {
                        const double a = exps[shell_exp_off[s] + k];
                        const double ek = coeffs[shell_coef_off[s] + k * nc + ci] *
                                          exp(-a * r2);
                        const double m = pow(d[0], e[0]) * pow(d[1], e[1]) * pow(d[2], e[2]);
                        val += ek * m;
                        for (int ax = 0; ax < 3; ++ax) {
                            /* d/dx [x^i ...] = (i x^(i-1) - 2 a x^(i+1)) ... */
                            double f = -2.0 * a * pow(d[ax], e[ax] + 1);
                            if (e[ax] > 0) f += e[ax] * pow(d[ax], e[ax] - 1);
                            double o = 1.0;
                            for (int bx = 0; bx < 3; ++bx)
                                if (bx != ax) o *= pow(d[bx], e[bx]);
                            gr[ax] += ek * f * o;
                        }
                    }
                    cart[0][c] = val;
                    cart[1][c] = gr[0]; cart[2][c] = gr[1]; cart[3][c] = gr[2];
                }
                for (int m = 0; m < ns; ++m)
                    for (int comp = 0; comp < 4; ++comp) {
                        double v = 0.0;
                        for (int c = 0; c < nca; ++c) v += b.c2s[l][c * ns + m] * cart[comp][c];
                        X[comp * plane + g * (int64_t)nao + ao[s] + ci * ns + m] = v;
                    }
            }
        }
    }
    free(ao);
    return 0;
}

int oracle_vv10_sum(const double* xyz, const double* q, const double* w0,
                    const double* kappa, int64_t n, double* F, double* U,
                    double* W) {
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n; ++i) {
        double f = 0.0, u = 0.0, w = 0.0;
        for (int64_t j = 0; j < n; ++j) {
            const double dx = xyz[3 * i] - xyz[3 * j], dy = xyz[3 * i + 1] - xyz[3 * j + 1],
                         dz = xyz[3 * i + 2] - xyz[3 * j + 2];
            const double r2 = dx * dx + dy * dy + dz * dz;
            const double g = r2 * w0[i] + kappa[i];
            const double gp = r2 * w0[j] + kappa[j];
            const double gt = g + gp;
            const double T = q[j] / (g * gp * gt);
            const double Tu = T * (1.0 / g + 1.0 / gt);
            f += T;
            u += Tu;
            w += Tu * r2;
        }
        F[i] = -1.5 * f;
        U[i] = u;
        W[i] = w;
    }
    return 0;
}

/* Becke fuzzy-cell weight of each point's owner atom (Becke 1988, three
 * smoothing iterations, no atomic size adjustment): the grid partition of
 * the synthetic workloads, for the CPU baselines that must not load the
 * product library.  Same formula as the product's grid builder. */
int oracle_becke_partition(const double* pts, int64_t n, const int* owner,
                           const double* atoms, int natm, double* out) {
    double* rinv = (double*)calloc((size_t)natm * natm, sizeof(double));
    if (!rinv) return 1;
    for (int a = 0; a < natm; ++a)
        for (int b = 0; b < natm; ++b) {
            if (a == b) continue;
            double d2 = 0.0;
            for (int x = 0; x < 3; ++x) {
                const double d = atoms[a * 3 + x] - atoms[b * 3 + x];
                d2 += d * d;
            }
            rinv[(size_t)a * natm + b] = 1.0 / sqrt(d2);
        }
    int fail = 0;
#pragma omp parallel
    {
        double* dist = (double*)malloc(sizeof(double) * (size_t)natm);
        double* P = (double*)malloc(sizeof(double) * (size_t)natm);
        if (!dist || !P) {
#pragma omp atomic write
            fail = 1;
        } else {
#pragma omp for schedule(static)
            for (int64_t i = 0; i < n; ++i) {
                for (int a = 0; a < natm; ++a) {
                    double d2 = 0.0;
                    for (int x = 0; x < 3; ++x) {
                        const double d = pts[i * 3 + x] - atoms[a * 3 + x];
                        d2 += d * d;
                    }
                    dist[a] = sqrt(d2);
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
        free(dist);
        free(P);
    }
    free(rinv);
    return fail;
}

/* ---- one-electron integrals and the Hartree potential (SCF oracle) ------ */

/* 1-D Hermite coefficients E[i][j][t] for i <= la, j <= lbx (lbx <= 5) */
#define EJX 6
#define ETX 10
static void hermite_ext(int la, int lbx, double p, double xpa, double xpb,
                        double E[LMAX + 1][EJX][ETX]) {
    memset(E, 0, sizeof(double) * (LMAX + 1) * EJX * ETX);
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
    for (int j = 1; j <= lbx; ++j)
        for (int i = 0; i <= la; ++i)
            for (int t = 0; t <= i + j; ++t) {
                double v = 0.0;
                if (t > 0) v += E[i][j - 1][t - 1] * inv2p;
                if (t <= i + j - 1) v += xpb * E[i][j - 1][t];
                if (t + 1 <= i + j - 1) v += (t + 1) * E[i][j - 1][t + 1];
                E[i][j][t] = v;
            }
}

/* Overlap S and kinetic T (nao, nao) in FP64 (Helgaker, Jorgensen, Olsen
 * ch. 9: S = K (pi/p)^(3/2) prod E^{ij}_0; the kinetic operator per axis
 * -2 b^2 S_(i,j+2) + b (2j+1) S_ij - j(j-1)/2 S_(i,j-2)). */
int oracle_int1e_st(OBASIS_ARGS, double* S, double* T) {
    obasis b;
    make_basis(&b, OBASIS_PASS);
    int* ao = ao_offsets(&b);
    const int nao = ao[nbas];
#pragma omp parallel for schedule(dynamic, 1)
    for (int ish = 0; ish < nbas; ++ish)
        for (int jsh = 0; jsh < nbas; ++jsh) {
            const int la = b.shell_l[ish], lb = b.shell_l[jsh];
            const int npi = b.shell_nprim[ish], npj = b.shell_nprim[jsh];
            const int nci = b.shell_nctr[ish], ncj = b.shell_nctr[jsh];
            const int nca = ncart(la), ncb = ncart(lb), nsa = nsph(la), nsb = nsph(lb);
            const double* A = b.atom_coords + 3 * b.shell_atom[ish];
            const double* B = b.atom_coords + 3 * b.shell_atom[jsh];
            double d2 = 0.0;
            for (int x = 0; x < 3; ++x) d2 += (A[x] - B[x]) * (A[x] - B[x]);
            for (int ci = 0; ci < nci; ++ci)
                for (int cj = 0; cj < ncj; ++cj) {
                    double cs[100], ct[100];
                    for (int q = 0; q < 100; ++q) cs[q] = ct[q] = 0.0;
                    for (int a = 0; a < npi; ++a)
                        for (int c = 0; c < npj; ++c) {
                            const double al = b.exps[b.shell_exp_off[ish] + a];
                            const double be = b.exps[b.shell_exp_off[jsh] + c];
                            const double p = al + be;
                            const double cc = b.coeffs[b.shell_coef_off[ish] + a * nci + ci] *
                                              b.coeffs[b.shell_coef_off[jsh] + c * ncj + cj] *
                                              exp(-al * be / p * d2);
                            double E[3][LMAX + 1][EJX][ETX];
                            for (int x = 0; x < 3; ++x) {
                                const double P = (al * A[x] + be * B[x]) / p;
                                hermite_ext(la, lb + 2, p, P - A[x], P - B[x], E[x]);
                            }
                            const double n3 = cc * pow(M_PI / p, 1.5);
                            for (int qa = 0; qa < nca; ++qa) {
                                int ia[3];
                                cart_comp(la, qa, &ia[0], &ia[1], &ia[2]);
                                for (int qb = 0; qb < ncb; ++qb) {
                                    int ib[3];
                                    cart_comp(lb, qb, &ib[0], &ib[1], &ib[2]);
                                    double s1[3], t1[3];
                                    for (int x = 0; x < 3; ++x) {
                                        const int i = ia[x], j = ib[x];
                                        s1[x] = E[x][i][j][0];
                                        t1[x] = -2.0 * be * be * E[x][i][j + 2][0] +
                                                be * (2 * j + 1) * E[x][i][j][0] -
                                                (j >= 2 ? 0.5 * j * (j - 1) * E[x][i][j - 2][0] : 0.0);
                                    }
                                    cs[qa * ncb + qb] += n3 * s1[0] * s1[1] * s1[2];
                                    ct[qa * ncb + qb] += n3 * (t1[0] * s1[1] * s1[2] +
                                                               s1[0] * t1[1] * s1[2] +
                                                               s1[0] * s1[1] * t1[2]);
                                }
                            }
                        }
                    for (int m1 = 0; m1 < nsa; ++m1)
                        for (int m2 = 0; m2 < nsb; ++m2) {
                            double vs = 0.0, vt = 0.0;
                            for (int qa = 0; qa < nca; ++qa)
                                for (int qb = 0; qb < ncb; ++qb) {
                                    const double w = b.c2s[la][qa * nsa + m1] *
                                                     b.c2s[lb][qb * nsb + m2];
                                    vs += w * cs[qa * ncb + qb];
                                    vt += w * ct[qa * ncb + qb];
                                }
                            const int64_t e = (int64_t)(ao[ish] + ci * nsa + m1) * nao +
                                              ao[jsh] + cj * nsb + m2;
                            S[e] = vs;
                            T[e] = vt;
                        }
                }
        }
    free(ao);
    return 0;
}

/* Hartree potential v[g] = sum_{mu nu} D_{mu nu} (mu nu | 1/|r - g|) at ng
 * points (absolute frame), every shell pair (no screening), FP64. */
int oracle_hartree(OBASIS_ARGS, const double* coords, int64_t ng, const double* D,
                   double* v) {
    obasis b;
    make_basis(&b, OBASIS_PASS);
    int* ao = ao_offsets(&b);
    const int nao = ao[nbas];
#pragma omp parallel for schedule(dynamic, 8)
    for (int64_t g = 0; g < ng; ++g) {
        double acc = 0.0;
        double A[16 * 16];
        for (int ish = 0; ish < nbas; ++ish)
            for (int jsh = 0; jsh <= ish; ++jsh) {
                int ni, nj;
                pair_block(&b, ish, jsh, coords + 3 * g, 0.0, A, &ni, &nj);
                const double w = ish == jsh ? 1.0 : 2.0;
                for (int m = 0; m < ni; ++m)
                    for (int n = 0; n < nj; ++n)
                        acc += w * D[(int64_t)(ao[ish] + m) * nao + ao[jsh] + n] *
                               A[m * 16 + n];
            }
        v[g] = acc;
    }
    free(ao);
    return 0;
}
