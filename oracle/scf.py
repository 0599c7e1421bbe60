"""FP64 host SCF of the wB97M-V / COSX(pjs) path -- the oracle of the
device SCF (pyscf_wb97mv_fast_gb300.scf).

TEST INFRASTRUCTURE ONLY: the checker of the GPU SCF (tests, the SCF
fixtures under tests/golden/ and the bench's parity fields).  Nothing in
the product imports it.

Every piece is FP64 and unscreened: S, T, V (oracle C); K(0) and K(omega)
as the reference's get_k builds them (oracle.cosx_k: F = X D, G = A F, K =
X^T (w o G), symmetrised); J = X^T (w o v_H) X with the analytic Hartree
potential v_H (oracle C); the semilocal functional on the XC grid; VV10 by
the brute-force double sum (oracle.nlc_vxc, the reference's VV10 flow,
gpu/vv10.py:268-342).  Pulay DIIS on the orthonormal-basis commutator, a
core-Hamiltonian start, convergence when |dE| and the commutator norm are
both small.  The functional is restated here from its published formulas
(short-range LDA exchange attenuation; VWN5 paramagnetic fit), not shared
with the product code.
"""
import math
import time

import numpy as np
from scipy.special import erf

import oracle

VWN5 = (0.0310907, -0.10498, 3.72744, 12.9352)      # A, x0, b, c (hartree)


def sr_lda_exchange(rho, omega):
    """Per-volume energy and potential of the erfc(omega r)/r-attenuated LDA
    exchange: e = e_x^LDA F(a), a = omega / (2 k_F) (closed form for a < 1.5,
    its asymptotic series above)."""
    r = np.maximum(rho, 1e-300)
    ex = -0.75 * (3.0 / math.pi) ** (1.0 / 3.0) * r ** (4.0 / 3.0)
    a = omega / (2.0 * (3.0 * math.pi ** 2 * r) ** (1.0 / 3.0))
    F = np.empty_like(a)
    dF = np.empty_like(a)
    lo = a < 1.5
    al = a[lo]
    e = np.exp(-1.0 / (4.0 * al * al))
    g = (math.sqrt(math.pi) * erf(1.0 / (2.0 * al)) + (2.0 * al - 4.0 * al ** 3) * e
         - 3.0 * al + 4.0 * al ** 3)
    F[lo] = 1.0 - 8.0 / 3.0 * al * g
    dF[lo] = -8.0 / 3.0 * (g + al * (12.0 * al * al * (1.0 - e) - 3.0))
    ah = a[~lo]
    coef = [1.0 / 36.0, -1.0 / 960.0, 1.0 / 26880.0, -1.0 / 829440.0,
            1.0 / 28385280.0, -1.0 / 1073479680.0, 1.0 / 44590694400.0,
            -1.0 / 2021444812800.0]
    F[~lo] = sum(c * ah ** (-2 * (k + 1)) for k, c in enumerate(coef))
    dF[~lo] = sum(-2.0 * (k + 1) * c * ah ** (-2 * (k + 1) - 1) for k, c in enumerate(coef))
    return ex * F, ex / r * (4.0 / 3.0 * F - a / 3.0 * dF)


def vwn5(rho):
    """Per-electron correlation energy and potential (VWN5, paramagnetic)."""
    A, x0, b, c = VWN5
    Q = math.sqrt(4.0 * c - b * b)
    x = np.sqrt((3.0 / (4.0 * math.pi * np.maximum(rho, 1e-300))) ** (1.0 / 3.0))
    X = x * x + b * x + c
    X0 = x0 * x0 + b * x0 + c
    at = np.arctan(Q / (2.0 * x + b))
    ec = A * (np.log(x * x / X) + 2.0 * b / Q * at - b * x0 / X0 *
              (np.log((x - x0) ** 2 / X) + 2.0 * (b + 2.0 * x0) / Q * at))
    d = (2.0 * x + b) ** 2 + Q * Q
    dec = A * (2.0 / x - (2.0 * x + b) / X - 4.0 * b / d - b * x0 / X0 *
               (2.0 / (x - x0) - (2.0 * x + b) / X - 4.0 * (b + 2.0 * x0) / d))
    return ec, ec - x / 6.0 * dec


class Functional:
    """alpha K(0) + beta K(omega) exact exchange, cx_sr SR-LDA exchange,
    VWN5 correlation, VV10 (b, C): the device SCF's stand-in functional."""

    def __init__(self, omega=0.3, alpha=0.15, beta=0.85, cx_sr=0.85, nlc=(6.0, 0.01)):
        self.omega, self.alpha, self.beta, self.cx_sr = omega, alpha, beta, cx_sr
        self.nlc = nlc

    def eval(self, rho):
        live = rho > 1e-14
        ex, vx = sr_lda_exchange(rho, self.omega)
        ec, vc = vwn5(rho)
        e = np.where(live, self.cx_sr * ex + rho * ec, 0.0)
        v = np.where(live, self.cx_sr * vx + vc, 0.0)
        return e, v


class HostScf:
    """The SCF on fixed grids (xc, sgx, nlc: objects with coords and
    weights in bohr; nlc may be None)."""

    def __init__(self, mol, grids, functional=None):
        self.mol = mol
        self.f = functional or Functional()
        self.g = grids
        S, T, V = oracle.int1e(mol)
        self.S, self.H = S, T + V
        s, U = np.linalg.eigh(S)
        keep = s > 1e-9
        self.Xo = U[:, keep] / np.sqrt(s[keep])[None, :]
        self.nocc = mol.nelectron // 2
        self.e_nuc = mol.energy_nuc()
        self.ao_xc = oracle.ao_eval(mol, grids['xc'].coords)
        self.ao_sgx = oracle.ao_eval(mol, grids['sgx'].coords)

    def fock(self, D):
        f, g = self.f, self.g
        K0 = oracle.cosx_k(self.mol, g['sgx'].coords, g['sgx'].weights, D, 0.0)
        Kw = oracle.cosx_k(self.mol, g['sgx'].coords, g['sgx'].weights, D, f.omega)
        Kx = f.alpha * K0 + f.beta * Kw
        vh = oracle.hartree(self.mol, g['sgx'].coords, D)
        X = self.ao_sgx
        J = X.T @ ((g['sgx'].weights * vh)[:, None] * X)
        X = self.ao_xc
        rho = ((X @ D) * X).sum(axis=1)
        e, v = f.eval(rho)
        exc = float((g['xc'].weights * e).sum())
        Vxc = X.T @ ((g['xc'].weights * v)[:, None] * X)
        enl, Vnl = 0.0, 0.0
        if g.get('nlc') is not None and f.nlc:
            _, enl, Vnl = oracle.nlc_vxc(self.mol, g['nlc'].coords, g['nlc'].weights, D,
                                         [(f.nlc, 1.0)])
        F = self.H + J - 0.5 * Kx + Vxc + Vnl
        E = (float((D * self.H).sum()) + 0.5 * float((D * J).sum())
             - 0.25 * float((D * Kx).sum()) + exc + enl + self.e_nuc)
        return E, 0.5 * (F + F.T)

    def diag(self, F):
        e, C = np.linalg.eigh(self.Xo.T @ F @ self.Xo)
        C = self.Xo @ C[:, :self.nocc]
        return 2.0 * C @ C.T

    def kernel(self, conv_tol=1e-11, conv_tol_grad=1e-7, max_cycle=100, space=8,
               verbose=False):
        D = self.diag(self.H)
        Fs, es = [], []
        e_last, hist = None, []
        t0 = time.perf_counter()
        for cycle in range(max_cycle):
            E, F = self.fock(D)
            FDS = F @ D @ self.S
            comm = self.Xo.T @ (FDS - FDS.T) @ self.Xo
            gn = float(np.linalg.norm(comm))
            dE = math.inf if e_last is None else abs(E - e_last)
            hist.append((E, dE, gn))
            if verbose:
                print('oracle cycle %2d E=%.12f dE=%.2e |g|=%.2e (%.0f s)'
                      % (cycle, E, dE, gn, time.perf_counter() - t0))
            if dE < conv_tol and gn < conv_tol_grad:
                return dict(e_tot=E, converged=True, cycles=cycle + 1, history=hist, dm=D)
            e_last = E
            Fs.append(F)
            es.append(comm)
            if len(Fs) > space:
                Fs.pop(0)
                es.pop(0)
            n = len(Fs)
            if n >= 2:
                B = np.zeros((n + 1, n + 1))
                for i in range(n):
                    for j in range(n):
                        B[i, j] = float((es[i] * es[j]).sum())
                B[:n, :n] /= B[:n, :n].diagonal().max()
                B[:n, n] = B[n, :n] = -1.0
                rhs = np.zeros(n + 1)
                rhs[n] = -1.0
                c = np.linalg.lstsq(B, rhs, rcond=None)[0][:n]
                F = sum(ci * Fi for ci, Fi in zip(c, Fs))
            D = self.diag(F)
        return dict(e_tot=hist[-1][0], converged=False, cycles=max_cycle, history=hist,
                    dm=D)
