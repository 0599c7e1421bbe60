"""Device-resident RKS SCF of the wB97M-V / COSX(pjs) hot path.

The reference runs its SCF through PySCF's loop on the host (scf.hf.kernel)
with the GPU K, XC and VV10 hooked in, staged by StagedSCF
(staging/schedule.py:99-485, run_staged :455-485): coarse grids and FP32 GPU
work early, fine grids and an FP64 tail late.  PySCF is not available on
these machines, so this module is the SCF loop itself, built from this
library's pieces and kept on the device from the first Fock build to the
converged energy:

    H = T + V                       wb_scf_int1e (FP64, once)
    K(0), K(omega)                  COSX multi-omega build: FP32 class
                                    kernels (mixed) or the plain FP64 form
    J = X^T (w o v_H) X             v_H from wb_hartree on the SGX grid
                                    (analytic potential, quadrature of
                                    mu nu v_H), FP32 or FP64
    E_xc, V_xc                      the functional on the XC grid
    E_nl, V_nl                      VV10 on the NLC grid (FP32 pair sum,
                                    FP64 elsewhere, as in the reference)
    F = H + J - K_x / 2 + V_xc + V_nl,  K_x = a K(0) + b K(omega)
    C from F C = S C e              FP64 eigensolver on the device
    CDIIS on the commutator X^T (F D S - S D F) X

and the energy
    E = tr(D H) + tr(D J)/2 - tr(D K_x)/4 + E_xc + E_nl + E_nuc.

Staging follows the reference's StagePlan (this package's
staging.schedule.StagePlan): S0 on coarse grids without VV10, S1 and S2 on
the final grids, then the FP64 tail (FP64 K, J and density GEMMs) from
which convergence is declared.  ``precision='fp64'`` runs the plain FP64
form on the final grids from the start: the comparison point of the
mixed-precision form and, checked against the oracle's SCF, the FP64
reference energy of molecules too large for the host oracle.

The semilocal functional is a stated stand-in: wB97M-V's pointwise
meta-GGA lives in libxc (third party, not on these machines).
``RshLdaVv10`` keeps wB97M-V's exact-exchange split (0.15 of the
full-range K plus 0.85 of the long-range K at omega = 0.3: short-range
0.15, long-range 1.0) and its VV10 parameters (b = 6.0, C = 0.01), with a
short-range LDA exchange (0.85) and VWN5 correlation for the semilocal
part.
"""
import math
import time

import numpy as np

from pyscf_wb97mv_fast_gb300.cosx import CosxEngine, as_molecule, round32
from pyscf_wb97mv_fast_gb300.staging.schedule import StagePlan


def _torch():
    import torch
    return torch


# -- the functional --------------------------------------------------------------

# large-a expansion of the short-range LDA exchange attenuation,
# F(a) = sum_k c_k a^(-2k), k = 1..8 (series of the closed form below)
_SR_SERIES = (1.0 / 36.0, -1.0 / 960.0, 1.0 / 26880.0, -1.0 / 829440.0,
              1.0 / 28385280.0, -1.0 / 1073479680.0, 1.0 / 44590694400.0,
              -1.0 / 2021444812800.0)
_VWN5 = dict(A=0.0310907, x0=-0.10498, b=3.72744, c=12.9352)


class RshLdaVv10:
    """Range-separated hybrid with wB97M-V's exact-exchange split and VV10.

    E_xc = -1/4 tr[D (alpha K(0) + beta K(omega))] + cx_sr E_x^{SR-LDA}(omega)
           + E_c^{VWN5} + E_nl^{VV10}(b, C)

    * the short-range LDA exchange per volume is e_x^LDA F(a),
      e_x^LDA = -3/4 (3/pi)^(1/3) rho^(4/3), a = omega / (2 k_F),
      k_F = (3 pi^2 rho)^(1/3),
      F(a) = 1 - 8/3 a [sqrt(pi) erf(1/(2a)) + (2a - 4a^3) exp(-1/(4a^2))
                        - 3a + 4a^3]
      (the erfc-attenuated uniform-gas exchange; its large-a series, eight
      terms, for a >= 1.5, where the closed form cancels: both are within
      5e-13 relative there);
    * VWN5: Vosko, Wilk, Nusair, Can. J. Phys. 58, 1200 (1980), the
      paramagnetic fit (A, x0, b, c) = (0.0310907, -0.10498, 3.72744,
      12.9352), hartree.
    """

    name = 'rsh-lda-vv10'

    def __init__(self, omega=0.3, alpha=0.15, beta=0.85, cx_sr=0.85,
                 nlc=(6.0, 0.01)):
        self.omega = float(omega)
        self.alpha = float(alpha)
        self.beta = float(beta)
        self.cx_sr = float(cx_sr)
        self.nlc = tuple(nlc) if nlc else None

    @property
    def omegas(self):
        return (0.0, self.omega)

    def eval(self, rho):
        """(e, v) per grid point for the density rho (torch FP64): e the
        semilocal energy per volume, v = de/drho."""
        torch = _torch()
        r = torch.clamp(rho, min=1e-300)
        live = rho > 1e-14
        ex_lda = -0.75 * (3.0 / math.pi) ** (1.0 / 3.0) * r ** (4.0 / 3.0)
        kf = (3.0 * math.pi ** 2 * r) ** (1.0 / 3.0)
        a = self.omega / (2.0 * kf)
        F, dF = _sr_attenuation(a)
        ex = ex_lda * F
        vx = (ex_lda / r) * (4.0 / 3.0 * F - a / 3.0 * dF)
        ec, vc = _vwn5(r)
        e = self.cx_sr * ex + r * ec
        v = self.cx_sr * vx + vc
        zero = torch.zeros_like(rho)
        return torch.where(live, e, zero), torch.where(live, v, zero)


def _sr_attenuation(a):
    torch = _torch()
    big = a >= 1.5
    a_s = torch.where(big, torch.ones_like(a), a)       # closed form branch
    b = 1.0 / (4.0 * a_s * a_s)
    eb = torch.exp(-b)
    g = (math.sqrt(math.pi) * torch.special.erf(1.0 / (2.0 * a_s))
         + (2.0 * a_s - 4.0 * a_s ** 3) * eb - 3.0 * a_s + 4.0 * a_s ** 3)
    dg = 12.0 * a_s * a_s * (1.0 - eb) - 3.0
    F_c = 1.0 - 8.0 / 3.0 * a_s * g
    dF_c = -8.0 / 3.0 * (g + a_s * dg)
    a_l = torch.where(big, a, 2.0 * torch.ones_like(a))   # series branch
    y = 1.0 / (a_l * a_l)
    F_s = torch.zeros_like(a)
    dF_s = torch.zeros_like(a)
    yk = torch.ones_like(a)
    for k, c in enumerate(_SR_SERIES, start=1):
        yk = yk * y
        F_s = F_s + c * yk
        dF_s = dF_s - 2.0 * k * c * yk / a_l
    return torch.where(big, F_s, F_c), torch.where(big, dF_s, dF_c)


def _vwn5(rho):
    """epsilon_c (per electron) and v_c of the paramagnetic VWN5 fit."""
    torch = _torch()
    A, x0, b, c = (_VWN5[k] for k in ('A', 'x0', 'b', 'c'))
    Q = math.sqrt(4.0 * c - b * b)
    X0 = x0 * x0 + b * x0 + c
    rs = (3.0 / (4.0 * math.pi * rho)) ** (1.0 / 3.0)
    x = torch.sqrt(rs)
    X = x * x + b * x + c
    at = torch.atan(Q / (2.0 * x + b))
    den = (2.0 * x + b) ** 2 + Q * Q
    ec = A * (torch.log(x * x / X) + 2.0 * b / Q * at
              - b * x0 / X0 * (torch.log((x - x0) ** 2 / X) + 2.0 * (b + 2.0 * x0) / Q * at))
    dec = A * (2.0 / x - (2.0 * x + b) / X - 4.0 * b / den
               - b * x0 / X0 * (2.0 / (x - x0) - (2.0 * x + b) / X
                                - 4.0 * (b + 2.0 * x0) / den))
    return ec, ec - x / 6.0 * dec


# -- grids -----------------------------------------------------------------------

class DeviceGrid:
    """One integration grid on the device: coordinates in the engine frame,
    weights, and the AO values (deriv 0, or 0 and 1), evaluated once."""

    def __init__(self, eng, grids, deriv=0):
        torch = _torch()
        self.level = getattr(grids, 'level', None)
        self.n = int(grids.weights.size)
        self.coords = eng.relative(np.asarray(grids.coords, dtype=np.float64))
        self.weights = torch.as_tensor(np.asarray(grids.weights, dtype=np.float64),
                                       device=eng.device)
        self.deriv = deriv
        if deriv == 0:
            self.X = eng.ao_eval(self.coords)             # (nao, ld)
        else:
            self.X = eng.ao_eval_deriv1(self.coords)      # (4, nao, ld)
        self.ld = int(self.X.shape[-1])
        w = torch.zeros(self.ld, dtype=torch.float64, device=eng.device)
        w[:self.n] = self.weights
        self.wpad = w


# -- the SCF -----------------------------------------------------------------------

DEFAULT_FINAL = dict(xc=2, sgx=1, nlc=1)
DEFAULT_COARSE = dict(xc=1, sgx=0)
# the reference's per-stage grid table (staging/schedule.py:91-96): S0, S1,
# S2 levels of the XC, SGX and NLC grids, None = VV10 off
REFERENCE_STAGE_LEVELS = dict(xc=(1, 3, 3), sgx=(1, 1, 2), nlc=(None, 1, 3))


def _gemm_mode(gemm):
    if gemm is True:
        return 'fp64'
    if gemm is False:
        return 'fp32'
    if gemm not in ('fp64', 'split64', 'fp32'):
        raise ValueError("gemm must be 'fp64', 'split64' or 'fp32'")
    return gemm


class DeviceRKS:
    """RKS SCF on one GPU for a Molecule (see the module docstring).

    ``levels`` are the final grid levels (xc, sgx, nlc; nlc None turns VV10
    off) and ``coarse`` those of stage S0 (xc, sgx; no VV10); S1 and S2 use
    the final grids.  ``stage_levels`` (kind -> (S0, S1, S2) levels, e.g.
    REFERENCE_STAGE_LEVELS, the reference's table in schedule.py:91-96)
    sets every stage's grids instead; the final grids are S2's.
    ``k_tile_tol`` is the COSX screen, ``j_tol`` the Hartree-potential
    screen.
    """

    def __init__(self, mol, functional=None, levels=None, coarse=None,
                 k_tile_tol=1e-11, j_tol=1e-14, device=None, verbose=False,
                 stage_levels=None):
        torch = _torch()
        self.mol = as_molecule(mol)
        self.functional = functional or RshLdaVv10()
        self.stage_levels = None
        if stage_levels is not None:
            if levels is not None or coarse is not None:
                raise ValueError('give stage_levels or levels/coarse, not both')
            self.stage_levels = {k: tuple(stage_levels[k]) for k in ('xc', 'sgx', 'nlc')}
            if any(len(v) != 3 for v in self.stage_levels.values()):
                raise ValueError('stage_levels: three levels (S0, S1, S2) per grid')
            levels = {k: v[2] for k, v in self.stage_levels.items()}
            coarse = {k: self.stage_levels[k][0] for k in ('xc', 'sgx')}
        self.levels = dict(DEFAULT_FINAL, **(levels or {}))
        self.coarse = dict(DEFAULT_COARSE, **(coarse or {}))
        self.k_tile_tol = float(k_tile_tol)
        self.j_tol = float(j_tol)
        self.verbose = verbose
        t0 = time.perf_counter()
        self.eng = CosxEngine(self.mol, device=device)
        self.device = self.eng.device
        S, T, V = self.eng.int1e()
        self.S = S
        self.H = T + V
        self.e_nuc = float(self.mol.energy_nuc())
        # canonical orthogonalisation X = U s^(-1/2) (s > 1e-9 kept)
        s, U = torch.linalg.eigh(S)
        keep = s > 1e-9
        self.Xo = U[:, keep] / torch.sqrt(s[keep])[None, :]
        self.nocc = self.mol.nelectron // 2
        self._grid_cache = {}
        self.profile = None           # dict of part -> seconds when profiling
        self._t_last = 0.0
        self.t_setup = time.perf_counter() - t0

    # -- pieces --------------------------------------------------------------
    def grid(self, kind, level):
        """DeviceGrid of kind 'xc' / 'sgx' (deriv 0) or 'nlc' (deriv 1)."""
        key = (kind, level)
        g = self._grid_cache.get(key)
        if g is None:
            from pyscf_wb97mv_fast_gb300.grids import build_grids
            g = DeviceGrid(self.eng, build_grids(self.mol, level=level),
                           deriv=1 if kind == 'nlc' else 0)
            g.level = level
            self._grid_cache[key] = g
        return g

    def _vmat(self, g, v, gemm):
        """X^T diag(w v) X over grid g (deriv-0 AO values), symmetric.
        gemm: 'fp64' (plain FP64 GEMM), 'split64' (the bf16 Ozaki split
        with the FP64 G = X v) or 'fp32' (the split with G rounded to
        FP32); True / False stand for 'fp64' / 'fp32'."""
        torch = _torch()
        gemm = _gemm_mode(gemm)
        X = g.X if g.deriv == 0 else g.X[0]
        if gemm == 'fp64':
            wv = torch.zeros(g.ld, dtype=torch.float64, device=self.device)
            wv[:g.n] = g.weights * v[:g.n]
            M = (X * wv[None, :]) @ X.T
        else:
            dt = torch.float32 if gemm == 'fp32' else torch.float64
            G = torch.zeros_like(X, dtype=dt)
            G[:, :g.n] = (X[:, :g.n] * v[None, :g.n]).to(dt)
            M = self.eng.ozaki_k(X, G, g.weights)
        return 0.5 * (M + M.T)

    def _density(self, g, D, gemm):
        torch = _torch()
        gemm = _gemm_mode(gemm)
        X = g.X if g.deriv == 0 else g.X[0]
        if gemm == 'fp64':
            T = D @ X
        elif gemm == 'split64':
            T = self.eng.ozaki_f(X, D, fp64=True)
        else:
            T = self.eng.ozaki_f(X, D).to(torch.float64)
        return (T * X).sum(dim=0)[:g.n]

    def k_matrices(self, D, g, fp64):
        om = self.functional.omegas
        if fp64:
            Kb = self.eng.get_k_fp64(g.coords, g.weights, D, om,
                                     tile_tol=self.k_tile_tol, stats=False)
        else:
            Kb = self.eng.get_k_multi(g.coords, g.weights, D, om,
                                      tile_tol=self.k_tile_tol, stats=False)
        return 0.5 * (Kb + Kb.transpose(1, 2))

    def vv10(self, D, g, gemm=True):
        """(E_nl, V_nl) on the NLC grid g (device scalars / matrix); gemm as
        for _vmat: the FP32 stages take its two GEMMs through the bf16
        split, the staged form's FP64 tail through the FP64 split."""
        from pyscf_wb97mv_fast_gb300.gpu.vv10 import vv10_energy_fock
        return vv10_energy_fock(self.eng, g, D, self.functional.nlc,
                                gemm=_gemm_mode(gemm))

    def _tick(self, name):
        """Per-part wall time (device-synchronised) when profiling."""
        if self.profile is None:
            return
        torch = _torch()
        torch.cuda.current_stream(self.device).synchronize()
        now = time.perf_counter()
        if name is not None:
            self.profile[name] = self.profile.get(name, 0.0) + now - self._t_last
        self._t_last = now

    def gemm_mode(self, fp64, inc32):
        """The quadrature-GEMM form of a Fock build (see fock)."""
        return 'fp32' if not fp64 else ('split64' if inc32 else 'fp64')

    def fock(self, D, grids, fp64, base=None, inc32=False, k=None, vv10=None):
        """(E, F, parts, base') for density D with grids = dict(xc=, sgx=,
        nlc=) DeviceGrids (nlc may be None).

        ``base`` (a dict of an earlier full build on the same grids and
        precision: D0, K_x0, J0, rho0) makes the build incremental from
        that fixed base, as a direct SCF's incremental Fock build:
        K_x = K_x0 + K_x(D - D0), its COSX screen running on F = X (D - D0),
        whose small entries drop most tasks.  With ``inc32`` (the staged
        form's FP64 tail) the increments of K_x, J and rho are built with
        the FP32 kernels: their rounding is ~1e-7 of the increment, itself
        small, so the operator stays FP64-accurate on the FP64 base; the
        tail's quadrature GEMMs (J, rho, V_xc, VV10) run through the FP64
        form of the bf16 split (42 bits of the row / column maxima, FP64
        operands and results).  Without it (the plain FP64 form) only K_x
        is incremental, in FP64, and every GEMM is a plain FP64 GEMM.
        base' is the base to keep (a new one after a full build).

        k (the symmetrised exchange matrices of D, or of D - base['D'] for
        an incremental build, built the way this build would) and vv10
        ((E_nl, V_nl) of D on the NLC grid) come from a batch of molecules
        (BatchedRKS) instead of being built here."""
        torch = _torch()
        f = self.functional
        gs, gx = grids['sgx'], grids['xc']
        gemm = self.gemm_mode(fp64, inc32)
        self._tick(None)
        full = base is None
        dD = None if full else D - base['D']
        if full:
            K = self.k_matrices(D, gs, fp64) if k is None else k
            Kx = f.alpha * K[0] + f.beta * K[1]
        else:
            dK = self.k_matrices(dD, gs, fp64 and not inc32) if k is None else k
            Kx = base['Kx'] + (f.alpha * dK[0] + f.beta * dK[1])
        self._tick('k')
        if full or not inc32:
            vh = self.eng.hartree(gs.coords, D, tol=self.j_tol, fp64=fp64)
            J = self._vmat(gs, vh, gemm)
        else:
            vh = self.eng.hartree(gs.coords, dD, tol=self.j_tol, fp64=False)
            J = base['J'] + self._vmat(gs, vh, 'fp32')
        self._tick('j')
        if full or not inc32:
            rho = self._density(gx, D, gemm)
        else:
            rho = base['rho'] + self._density(gx, dD, 'fp32')
        e, v = f.eval(rho)
        exc = (gx.weights * e).sum()
        Vxc = self._vmat(gx, v, gemm)
        self._tick('xc')
        if vv10 is not None:
            enl, Vnl = vv10
        elif grids.get('nlc') is not None and f.nlc:
            enl, Vnl = self.vv10(D, grids['nlc'], gemm)
        else:
            enl, Vnl = torch.zeros((), dtype=torch.float64, device=self.device), 0.0
        self._tick('vv10')
        F = self.H + J - 0.5 * Kx + Vxc + Vnl
        e1 = (D * self.H).sum()
        ej = 0.5 * (D * J).sum()
        ek = -0.25 * (D * Kx).sum()
        E = e1 + ej + ek + exc + enl + self.e_nuc
        new_base = dict(D=D, Kx=Kx, J=J, rho=rho) if full else base
        return E, F, dict(e1=e1, ej=ej, ek=ek, exc=exc, enl=enl), new_base

    def _diag(self, F):
        torch = _torch()
        Fo = self.Xo.T @ F @ self.Xo
        e, Co = torch.linalg.eigh(Fo)
        C = self.Xo @ Co
        Cocc = C[:, :self.nocc]
        return 2.0 * Cocc @ Cocc.T, e

    def _commutator(self, F, D):
        FDS = F @ D @ self.S
        return self.Xo.T @ (FDS - FDS.T) @ self.Xo

    def core_guess(self):
        return self._diag(self.H)[0]

    # -- the loop --------------------------------------------------------------
    def kernel(self, precision='mixed', dm0=None, conv_tol=1e-9, conv_tol_grad=1e-5,
               max_cycle=80, diis_space=8, plan=None, reference_energy=None,
               incremental=True, rebuild_every=None, profile=False):
        """Run the SCF; returns a dict with e_tot, converged, cycles, wall
        (seconds, device-synchronised), per-cycle history and, for the
        staged form, the energy at the end of each stage.  precision:
        'mixed' (staged, FP32 GPU work, FP64 tail) or 'fp64' (the plain FP64
        form on the final grids).  incremental: after a full FP64 build the
        next FP64 cycles build from it as a fixed base (``fock``): the
        staged form's tail adds FP32 increments of K, J and rho, the plain
        FP64 form FP64 increments of K; a full rebuild at every stage or
        precision switch (the reference forces that rebuild on its
        switches, staging/schedule.py:335-346) and every rebuild_every
        cycles -- by default 8 for the plain FP64 form, as PySCF's direct
        SCF does, and never for the staged form's tail, whose increments
        are built afresh each cycle from its one FP64 base (a rebuild there
        only re-draws the screening error, about 1e-8 Ha on C20H42, and
        costs a full FP64 exchange build).  FP32 stages always build in
        full.
        profile: per-part seconds in out['profile'] (synchronises)."""
        torch = _torch()
        # the current stream only: solves on other streams keep running
        stream = torch.cuda.current_stream(self.device)
        stream.synchronize()
        run = ScfRun(self, precision, dm0, conv_tol, conv_tol_grad, max_cycle,
                     diis_space, plan, reference_energy, incremental, rebuild_every)
        self.profile = {} if profile else None
        while not run.done:
            req = run.request()
            E, F, parts, base = self.fock(run.D, req['grids'], req['fp64'],
                                          base=req['base'], inc32=run.staged)
            run.advance(E, F, parts, base)
        stream.synchronize()
        out = run.result()
        if self.profile is not None:
            out['profile'] = dict(self.profile)
            self.profile = None
        return out

    def _stage_grids(self, stage):
        if self.stage_levels is not None:
            lv = {k: v[stage] for k, v in self.stage_levels.items()}
            return dict(xc=self.grid('xc', lv['xc']), sgx=self.grid('sgx', lv['sgx']),
                        nlc=None if lv['nlc'] is None else self.grid('nlc', lv['nlc']))
        if stage == 0:
            return dict(xc=self.grid('xc', self.coarse['xc']),
                        sgx=self.grid('sgx', self.coarse['sgx']), nlc=None)
        nlc = self.levels['nlc']
        return dict(xc=self.grid('xc', self.levels['xc']),
                    sgx=self.grid('sgx', self.levels['sgx']),
                    nlc=None if nlc is None else self.grid('nlc', nlc))


class ScfRun:
    """One SCF between its Fock builds: the loop of DeviceRKS.kernel cut
    where the builds of several molecules can be shared (BatchedRKS steps
    many runs at once).  request() names this cycle's build; advance()
    takes its result (E, F) and does the rest of the cycle: the
    commutator, the convergence test, the stage plan's switches, DIIS and
    the diagonalisation.  The caller synchronises the device before
    construction (the wall clock starts there)."""

    def __init__(self, rks, precision='mixed', dm0=None, conv_tol=1e-9,
                 conv_tol_grad=1e-5, max_cycle=80, diis_space=8, plan=None,
                 reference_energy=None, incremental=True, rebuild_every=None):
        torch = _torch()
        if precision not in ('mixed', 'fp64'):
            raise ValueError("precision must be 'mixed' or 'fp64'")
        if rebuild_every is None:
            rebuild_every = 8 if precision == 'fp64' else 1 << 30
        self.t0 = time.perf_counter()
        self.rks = rks
        self.precision = precision
        self.staged = precision == 'mixed'
        self.plan = None
        if self.staged:
            self.plan = plan or StagePlan(fp64_final=True, tau_fp64=1e-6,
                                          tau_fp64_g=1e-4)
        self.D = rks.core_guess() if dm0 is None else torch.as_tensor(
            dm0, dtype=torch.float64, device=rks.device)
        self.stage, self.fp64 = (0, False) if self.staged else (2, True)
        self.diis_space = diis_space
        self.diis = _Cdiis(diis_space)
        self.hist, self.stage_end = [], []
        self.e_last, self.converged, self.done = None, False, False
        self.base, self.since_full, self._use = None, 0, None
        self.conv_tol, self.conv_tol_grad = conv_tol, conv_tol_grad
        self.max_cycle = int(max_cycle)
        self.incremental, self.rebuild_every = bool(incremental), int(rebuild_every)
        self.reference_energy = reference_energy
        self.cycle = 0
        self.parts = {}
        self.done = self.max_cycle <= 0

    def request(self):
        """This cycle's build: grids, fp64, the incremental base (or None),
        and the exchange build it needs -- k_mode 'fp32' (the FP32 class
        kernels) or 'fp64' (the plain FP64 form) of k_dm, the density for a
        full build or its change from the base for an incremental one."""
        grids = self.rks._stage_grids(self.stage)
        use = (self.base if self.incremental and self.fp64
               and self.since_full < self.rebuild_every else None)
        self._use = use
        if use is None:
            k_mode, k_dm = ('fp64' if self.fp64 else 'fp32'), self.D
        else:
            k_mode = 'fp64' if (self.fp64 and not self.staged) else 'fp32'
            k_dm = self.D - use['D']
        return dict(grids=grids, fp64=self.fp64, base=use, k_mode=k_mode, k_dm=k_dm,
                    gemm=self.rks.gemm_mode(self.fp64, self.staged))

    def advance(self, E, F, parts, base):
        torch = _torch()
        rks = self.rks
        self.base = base
        self.since_full = 1 if self._use is None else self.since_full + 1
        self.parts = parts
        comm = rks._commutator(F, self.D)
        gnorm = float(torch.linalg.norm(comm))
        Ef = float(E)
        dE = math.inf if self.e_last is None else abs(Ef - self.e_last)
        cycle = self.cycle
        self.cycle += 1
        self.hist.append(dict(cycle=cycle, stage=self.stage, fp64=self.fp64, e=Ef,
                              dE=dE, gnorm=gnorm, t=time.perf_counter() - self.t0))
        if rks.verbose:
            print('cycle %2d S%d %s E=%.12f dE=%.2e |g|=%.2e'
                  % (cycle, self.stage, 'fp64' if self.fp64 else 'fp32', Ef, dE, gnorm))
        may_stop = (not self.staged) or self.plan.may_converge
        if may_stop and dE < self.conv_tol and gnorm < self.conv_tol_grad:
            self.converged = self.done = True
            return
        decision = self.plan.after_cycle(dE, gnorm) if self.staged else None
        if decision is not None:
            self.stage_end.append(dict(stage=self.stage, fp64=self.fp64, e=Ef,
                                       cycles=cycle + 1))
            if decision[0] == 'stage':
                self.stage = decision[1]
            else:
                self.fp64 = True
            self.diis = _Cdiis(self.diis_space)      # the functional changed
            self.e_last = None
            self.base = None                         # full rebuild after a switch
            self.D = rks._diag(F)[0]
        else:
            self.e_last = Ef
            Fd = self.diis.update(F, comm)
            self.D = rks._diag(Fd)[0]
        if self.cycle >= self.max_cycle:
            self.done = True

    def result(self):
        """The run's result dict (wall from construction to now)."""
        wall = time.perf_counter() - self.t0
        hist = self.hist
        out = dict(e_tot=hist[-1]['e'] if hist else None, converged=self.converged,
                   cycles=len(hist), wall=wall, setup_s=self.rks.t_setup, history=hist,
                   precision=self.precision, stages=self.stage_end,
                   parts={k: float(v) for k, v in self.parts.items()}, dm=self.D,
                   incremental=self.incremental)
        ref = self.reference_energy
        if ref is not None and hist:
            out['error_vs_reference'] = out['e_tot'] - float(ref)
            for h in hist:
                h['err'] = h['e'] - float(ref)
            for st in self.stage_end:
                st['err'] = st['e'] - float(ref)
        return out


class _Cdiis:
    """Pulay's commutator DIIS on the device (P. Pulay, J. Comput. Chem. 3,
    556 (1982)): extrapolated F = sum c_i F_i with sum c_i = 1 minimising
    |sum c_i e_i|, e_i the orthonormal-basis commutators."""

    def __init__(self, space=8):
        self.space = int(space)
        self.F, self.e = [], []

    def update(self, F, e):
        torch = _torch()
        self.F.append(F)
        self.e.append(e)
        if len(self.F) > self.space:
            self.F.pop(0)
            self.e.pop(0)
        n = len(self.F)
        if n < 2:
            return F
        E = torch.stack([x.reshape(-1) for x in self.e])
        B = torch.zeros((n + 1, n + 1), dtype=torch.float64, device=F.device)
        B[:n, :n] = E @ E.T
        B[:n, n] = -1.0
        B[n, :n] = -1.0
        rhs = torch.zeros(n + 1, dtype=torch.float64, device=F.device)
        rhs[n] = -1.0
        scale = B[:n, :n].diagonal().max()
        if scale > 0:
            B[:n, :n] /= scale
        # the (n+1)-square system is solved on the host (least squares: the
        # error vectors can be nearly dependent)
        c = np.linalg.lstsq(B.cpu().numpy(), rhs.cpu().numpy(), rcond=None)[0][:n]
        out = torch.zeros_like(F)
        for ci, Fi in zip(c, self.F):
            out += float(ci) * Fi
        return out


class BatchedRKS:
    """The SCFs of several molecules in lockstep on one GPU.  Every cycle
    the exchange builds that run on the FP32 class kernels -- the FP32
    stages' full builds and the FP64 tail's increments -- of all molecules
    are one batched build (CosxBatch: one launch per class kernel over the
    molecules, per SGX grid level), and the VV10 double sums of all
    molecules one launch (Vv10Kernel.kernel_sum_batch); the plain-FP64
    exchange builds (the tail's full bases), J, the semilocal XC, Fock
    assembly, DIIS and the diagonalisation run per molecule.  Each molecule
    follows its own stage plan and stops at its own convergence; a
    molecule that is done, or whose build this cycle is not batched, is
    left out of the batch run.  The batched builds are bitwise the
    per-molecule ones, so each molecule's SCF is the one DeviceRKS runs
    alone.  The arguments after mols are those of DeviceRKS, for every
    molecule."""

    def __init__(self, mols, functional=None, levels=None, coarse=None,
                 k_tile_tol=1e-11, j_tol=1e-14, device=None, stage_levels=None):
        if not mols:
            raise ValueError('no molecule')
        self.rks = [DeviceRKS(m, functional, levels, coarse, k_tile_tol, j_tol,
                              device=device, stage_levels=stage_levels) for m in mols]
        self.k_tile_tol = float(k_tile_tol)
        self._kb = {}

    def _k_batch(self, level):
        """The batched exchange build on the SGX grids of one level (its own
        engines: a batch owns its engines' workspaces while it lives)."""
        from pyscf_wb97mv_fast_gb300.cosx import CosxBatch, CosxEngine
        b = self._kb.get(level)
        if b is None:
            engines = [CosxEngine(r.mol, device=r.device) for r in self.rks]
            grids = []
            for r in self.rks:
                g = r.grid('sgx', level)
                grids.append((g.coords, g.weights))
            b = CosxBatch(engines, grids, self.rks[0].functional.omegas,
                          tile_tol=self.k_tile_tol)
            self._kb[level] = b
        return b

    def kernel(self, precision='mixed', reference_energies=None, **kw):
        """Run every molecule's SCF (precision and the keywords of
        DeviceRKS.kernel, for every molecule); returns one result dict per
        molecule, plus out-of-band 'wall' (the whole batch) in each."""
        from pyscf_wb97mv_fast_gb300.gpu.vv10 import Vv10Kernel, vv10_finish, vv10_prepare
        torch = _torch()
        dev = self.rks[0].device
        stream = torch.cuda.current_stream(dev)
        stream.synchronize()
        t0 = time.perf_counter()
        refs = reference_energies or [None] * len(self.rks)
        runs = [ScfRun(r, precision, reference_energy=e, **kw)
                for r, e in zip(self.rks, refs)]
        vv = Vv10Kernel(0.0)
        n = len(runs)
        batched_builds = 0
        while not all(r.done for r in runs):
            act = [i for i in range(n) if not runs[i].done]
            req = {i: runs[i].request() for i in act}
            # exchange: the FP32-kernel builds batched per SGX level
            K = {}
            by_level = {}
            for i in act:
                if req[i]['k_mode'] == 'fp32':
                    by_level.setdefault(req[i]['grids']['sgx'].level, []).append(i)
                else:
                    K[i] = self.rks[i].k_matrices(req[i]['k_dm'], req[i]['grids']['sgx'],
                                                  True)
            for level, idx in by_level.items():
                qds = [req[i]['k_dm'] if i in idx else None for i in range(n)]
                out = self._k_batch(level).run(qds)
                batched_builds += 1
                for i in idx:
                    K[i] = 0.5 * (out[i] + out[i].transpose(1, 2))
            # VV10: the double sums of every molecule with an NLC grid in one
            # launch
            st = {}
            for i in act:
                r = self.rks[i]
                g = req[i]['grids'].get('nlc')
                if g is not None and r.functional.nlc:
                    st[i] = vv10_prepare(r.eng, g, runs[i].D, r.functional.nlc,
                                         req[i]['gemm'])
            V = {}
            if st:
                idx = sorted(st)
                F, U, W = vv.kernel_sum_batch([st[i]['xyz'] for i in idx],
                                              [st[i]['q'] for i in idx],
                                              [st[i]['W0'] for i in idx],
                                              [st[i]['kappa'] for i in idx])
                for j, i in enumerate(idx):
                    V[i] = vv10_finish(st[i], F[j], U[j], W[j])
            for i in act:
                r = self.rks[i]
                E, Fk, parts, base = r.fock(runs[i].D, req[i]['grids'], req[i]['fp64'],
                                            base=req[i]['base'], inc32=runs[i].staged,
                                            k=K[i], vv10=V.get(i))
                runs[i].advance(E, Fk, parts, base)
        stream.synchronize()
        wall = time.perf_counter() - t0
        outs = [r.result() for r in runs]
        for o in outs:
            o['batch_wall'] = wall
            o['batched_exchange_builds'] = batched_builds
        return outs

    def close(self):
        """Frees the batched builds, the engines they own (one per molecule
        and grid level, destroyed after their batch) and every molecule's
        own engine."""
        for b in self._kb.values():
            b.close()
            for e in b.engines:
                e.close()
        self._kb = {}
        for r in self.rks:
            r.eng.close()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

