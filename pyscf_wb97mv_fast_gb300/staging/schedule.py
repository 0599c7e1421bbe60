"""Staged SCF driver: coarse grids and FP32 GPU work early, fine grids and an
FP64 tail late (reference: pyscf_wb97mv_fast/staging/schedule.py:99-485).

Three stages.  Every switch changes the grids, drops the DIIS history and
forces the next Fock build to be a full one (no incremental J/K against the
previous density); inside a stage nothing changes.

    stage  entered when                   XC level  VV10          SGX level
    S0     at the start                   1         off           1
    S1     |g| < tau1   (1e-3)            3         on, level 1   1
    S2     |dE| < tau2  (1e-6 Ha)         3         on, level 3   2

(|g| < tau2_g is an optional extra gate for S1 -> S2, off by default; S1 is
left after max_s1_cycles in any case.)

Precision.  ``gpu_stages`` lists the stages whose K/VV10 run through
``install_gpu`` (FP32 fused kernels on the GPU); the other stages run the
stock PySCF FP64 code.  With ``fp64_final=True`` (needs 2 in gpu_stages)
S2 starts on the GPU and, once |dE| < tau_fp64 and |g| < tau_fp64_g (or
after max_fp32_s2_cycles), the GPU hooks come off for the remaining cycles
-- again with a DIIS reset and a full Fock rebuild, since the energy
functional changes by the FP32 error -- and convergence is never declared
before that switch.  ``fp64_final_vv10='gpu'`` keeps VV10 (only) on the GPU
for the FP64 tail; ``'cpu'`` moves it back too.  ``fp64_final_k='gpu'``
(an addition; the reference's tail always runs K on the CPU) keeps K on
the GPU for the tail in its plain FP64 form (``k_precision='fp64'``).  ``fp64_conv_tol`` is the
|dE| threshold of the FP64 tail alone (the |g| threshold stays
conv_tol_grad or sqrt(conv_tol)); setting it also turns mf.conv_check off
while attached.

Two more switches: ``vv10_mode='nonscf'`` keeps VV10 off for the whole SCF
and adds one VV10 energy on the final density afterwards
(``add_nonscf_vv10``); ``s2_mode='steps'`` stops after ``s2_steps`` S2
cycles instead of converging (mf.conv_check off while attached).

The switching rules live in ``StagePlan``, which knows nothing of PySCF;
``StagedSCF`` applies its decisions to an RKS/COSX mf through the two hooks
PySCF's SCF loop offers (``mf.callback`` after each cycle and
``mf.check_convergence``), and undoes every change on ``restore()``:

    mf = dft.RKS(mol, xc='wb97m-v').COSX(pjs=True)
    with StagedSCF(mf, gpu_stages=(0, 1, 2), fp64_final=True) as staged:
        mf.kernel()
    info = staged.info()

Importing this module does not import PySCF.
"""
import math
import sys
import time

from pyscf_wb97mv_fast_gb300.core.hooks import HookSet, reset_diis

STAGE_NAMES = ('S0', 'S1', 'S2')

DEFAULT_TAU1 = 1e-3           # |g| gate S0 -> S1
DEFAULT_TAU2 = 1e-6           # |dE| gate S1 -> S2 (Ha)
DEFAULT_XC_LEVELS = (1, 3, 3)
DEFAULT_NLC_LEVELS = (None, 1, 3)    # None: VV10 off in that stage
DEFAULT_SGX_LEVELS = (1, 1, 2)


class StagePlan:
    """Stage and precision decisions from the per-cycle |dE| and |g|.

    ``after_cycle(dE, gnorm)`` is called once per finished SCF cycle and
    returns None, ``('stage', new_stage, forced)`` or ``('fp64', forced)``;
    at most one decision per cycle, a stage switch taking precedence
    (reference schedule.py:306-367).  ``may_converge`` is False while an
    FP64 tail is still due.
    """

    def __init__(self, tau1=DEFAULT_TAU1, tau2=DEFAULT_TAU2,
                 tau2_g=math.inf, max_s1_cycles=8, fp64_final=False,
                 tau_fp64=None, tau_fp64_g=5e-5, max_fp32_s2_cycles=8):
        self.tau1 = float(tau1)
        self.tau2 = float(tau2)
        self.tau2_g = float(tau2_g)
        self.max_s1_cycles = int(max_s1_cycles)
        self.fp64_final = bool(fp64_final)
        self.tau_fp64 = float(self.tau2 if tau_fp64 is None else tau_fp64)
        self.tau_fp64_g = float(tau_fp64_g)
        self.max_fp32_s2_cycles = int(max_fp32_s2_cycles)
        self.reset()

    def reset(self):
        self.stage = 0
        self.fp64_phase = False
        self.s1_cycles = 0
        self.fp32_s2_cycles = 0

    @property
    def may_converge(self):
        return not (self.fp64_final and not self.fp64_phase)

    def after_cycle(self, dE, gnorm):
        if self.stage == 1:
            self.s1_cycles += 1
        decision = None
        if self.stage == 0 and gnorm < self.tau1:
            decision = ('stage', 1, False)
        elif self.stage == 1 and dE < self.tau2 and gnorm < self.tau2_g:
            decision = ('stage', 2, False)
        elif self.stage == 1 and self.s1_cycles >= self.max_s1_cycles:
            decision = ('stage', 2, True)
        fp32_s2 = self.stage == 2 and not self.fp64_phase
        if fp32_s2:
            self.fp32_s2_cycles += 1
        if decision is not None:
            self.stage = decision[1]
            return decision
        if self.fp64_final and fp32_s2:
            if dE < self.tau_fp64 and gnorm < self.tau_fp64_g:
                decision = ('fp64', False)
            elif self.fp32_s2_cycles >= self.max_fp32_s2_cycles:
                decision = ('fp64', True)
            if decision is not None:
                self.fp64_phase = True
        return decision


def _note(mf, fmt, *args):
    """PySCF-style NOTE-level log line (verbose >= 3) on mf.stdout."""
    if getattr(mf, 'verbose', 0) >= 3:
        out = getattr(mf, 'stdout', None) or sys.stdout
        out.write((fmt % args) + '\n')


def _default_installer(mf, **kwargs):
    from pyscf_wb97mv_fast_gb300.gpu.install import install_gpu
    return install_gpu(mf, **kwargs)


class StagedSCF:
    """Attach to an RKS/COSX mf to run its SCF in stages (context manager).

    The keyword names, defaults and errors are the reference's
    (schedule.py:108-183).  ``installer(mf, **gpu_kwargs) -> HookSet``
    installs the GPU hooks of a GPU stage (default: ``install_gpu``).
    ``restore()`` undoes every attribute change; the grids stay built at
    the last stage's level, as a plain SCF leaves them.
    """

    def __init__(self, mf, tau1=DEFAULT_TAU1, tau2=DEFAULT_TAU2,
                 xc_levels=DEFAULT_XC_LEVELS, nlc_levels=DEFAULT_NLC_LEVELS,
                 sgx_levels=DEFAULT_SGX_LEVELS,
                 vv10_mode='late_scf', s2_mode='converge', s2_steps=1,
                 nlc_production_level=3, gpu_stages=(), gpu_kwargs=None,
                 fp64_final=False, tau_fp64=None, fp64_final_vv10='gpu',
                 tau_fp64_g=5e-5, max_fp32_s2_cycles=8, tau2_g=math.inf,
                 max_s1_cycles=8, fp64_conv_tol=None, installer=None,
                 fp64_final_k='cpu'):
        df = getattr(mf, 'with_df', None)
        if df is None or not hasattr(df, 'grids_level_i'):
            raise TypeError('StagedSCF needs a COSX (SGX) mf, got %s'
                            % type(mf))
        if not set(gpu_stages) <= {0, 1, 2}:
            raise ValueError('gpu_stages entries must be stage indices 0, 1, 2')
        if fp64_final and 2 not in gpu_stages:
            raise ValueError('fp64_final switches precision inside S2: '
                             'needs 2 in gpu_stages')
        if fp64_final_vv10 not in ('gpu', 'cpu'):
            raise ValueError("fp64_final_vv10 must be 'gpu' or 'cpu'")
        if fp64_final_k not in ('gpu', 'cpu'):
            raise ValueError("fp64_final_k must be 'gpu' or 'cpu'")
        if fp64_conv_tol is not None and not fp64_final:
            raise ValueError('fp64_conv_tol applies to the FP64 tail: '
                             'needs fp64_final=True')
        if vv10_mode not in ('late_scf', 'nonscf'):
            raise ValueError("vv10_mode must be 'late_scf' or 'nonscf'")
        if s2_mode not in ('converge', 'steps'):
            raise ValueError("s2_mode must be 'converge' or 'steps'")
        for name, levels in (('xc_levels', xc_levels),
                             ('nlc_levels', nlc_levels),
                             ('sgx_levels', sgx_levels)):
            if len(levels) != 3:
                raise ValueError('%s needs 3 entries (S0, S1, S2)' % name)
        self.mf = mf
        self.xc_levels = tuple(xc_levels)
        self.nlc_levels = tuple(nlc_levels)
        self.sgx_levels = tuple(sgx_levels)
        self.vv10_mode = vv10_mode
        self.s2_mode = s2_mode
        self.s2_steps = int(s2_steps)
        self.nlc_production_level = int(nlc_production_level)
        self.gpu_stages = tuple(sorted(set(gpu_stages)))
        self.gpu_kwargs = dict(gpu_kwargs or {})
        self.fp64_final_vv10 = fp64_final_vv10
        self.fp64_final_k = fp64_final_k
        self.fp64_conv_tol = (None if fp64_conv_tol is None
                              else float(fp64_conv_tol))
        self.plan = StagePlan(tau1=tau1, tau2=tau2, tau2_g=tau2_g,
                              max_s1_cycles=max_s1_cycles,
                              fp64_final=fp64_final, tau_fp64=tau_fp64,
                              tau_fp64_g=tau_fp64_g,
                              max_fp32_s2_cycles=max_fp32_s2_cycles)
        self._installer = installer or _default_installer
        self.s2_cycles = 0
        self.switches = []
        self.history = []
        self._hooks = None
        self._gpu_hooks = None
        self._attached = False
        self._t_attach = None
        self._saved = None

    # the reference exposes these as attributes
    tau1 = property(lambda self: self.plan.tau1)
    tau2 = property(lambda self: self.plan.tau2)
    tau2_g = property(lambda self: self.plan.tau2_g)
    tau_fp64 = property(lambda self: self.plan.tau_fp64)
    tau_fp64_g = property(lambda self: self.plan.tau_fp64_g)
    fp64_final = property(lambda self: self.plan.fp64_final)
    stage = property(lambda self: self.plan.stage)
    fp64_phase = property(lambda self: self.plan.fp64_phase)

    @property
    def stage_name(self):
        return STAGE_NAMES[self.plan.stage]

    # -- attach / restore ----------------------------------------------------
    def __enter__(self):
        return self.attach()

    def __exit__(self, *exc):
        self.restore()

    def attach(self):
        """Pin the S0 settings and hook the callback and convergence test."""
        if self._attached:
            raise RuntimeError('StagedSCF already attached')
        mf, df = self.mf, self.mf.with_df
        self._saved = dict(nlc=mf.nlc, conv_check=mf.conv_check,
                           grids_level=mf.grids.level,
                           nlcgrids_level=mf.nlcgrids.level,
                           sgx_levels=(df.grids_level_i, df.grids_level_f))
        if self.s2_mode == 'steps' or self.fp64_conv_tol is not None:
            # no stock extra cycle after convergence: it would be one more
            # full cycle past the stage's own stopping rule
            mf.conv_check = False
        self._hooks = HookSet()
        self._hooks.wrap(mf, 'callback', self._make_callback)
        self._hooks.wrap(mf, 'check_convergence', self._make_conv_check)
        self.plan.reset()
        self.s2_cycles = 0
        self._apply_stage(0)
        self._attached = True
        self._t_attach = time.perf_counter()
        _note(mf, 'StagedSCF attached, stage S0 (vv10_mode=%s s2_mode=%s)',
              self.vv10_mode, self.s2_mode)
        return self

    def restore(self):
        """Undo every attribute change (no-op when not attached)."""
        if not self._attached:
            return
        mf, df, s = self.mf, self.mf.with_df, self._saved
        self._hooks.restore_all()
        self._set_gpu(False)
        mf.nlc = s['nlc']
        mf.conv_check = s['conv_check']
        mf.grids.level = s['grids_level']
        mf.nlcgrids.level = s['nlcgrids_level']
        df.grids_level_i, df.grids_level_f = s['sgx_levels']
        self._attached = False

    # -- the two SCF-loop hooks ----------------------------------------------
    def _make_callback(self, prev):
        def callback(envs):
            self._on_cycle_end(envs)
            if callable(prev):
                prev(envs)
        return callback

    def _make_conv_check(self, user_check):
        """Replaces PySCF's convergence branch, so without a user
        check_convergence it restates the stock test: |dE| < conv_tol and
        |g| < conv_tol_grad (default sqrt(conv_tol)); on the extra
        conv_check cycle -- the second call with the same cycle number --
        |dE| < 10 conv_tol or |g| < 3 conv_tol_grad (reference
        schedule.py:250-294)."""
        mf = self.mf
        last = {'cycle': None}

        def check_convergence(envs):
            if not self.plan.may_converge:
                return False
            if self.plan.stage == 2:
                self.s2_cycles += 1
                if self.s2_mode == 'steps' and self.s2_cycles >= self.s2_steps:
                    return True
            if callable(user_check):
                return user_check(envs)
            tol = mf.conv_tol
            tol_g = mf.conv_tol_grad
            if tol_g is None:
                tol_g = math.sqrt(tol)
            if self.plan.fp64_phase and self.fp64_conv_tol is not None:
                tol = self.fp64_conv_tol
            cycle = envs.get('cycle')
            repeat = cycle is not None and cycle == last['cycle']
            last['cycle'] = cycle
            dE = abs(envs['e_tot'] - envs['last_hf_e'])
            g = envs['norm_gorb']
            if repeat:
                return dE < tol * 10 or g < tol_g * 3
            return dE < tol and g < tol_g
        return check_convergence

    def _on_cycle_end(self, envs):
        t = time.perf_counter()
        cycle = int(envs.get('cycle', -1))
        g = float(envs.get('norm_gorb', math.nan))
        e_tot = float(envs.get('e_tot', math.nan))
        dE = abs(e_tot - float(envs.get('last_hf_e', math.nan)))
        rec = dict(cycle=cycle, stage=self.plan.stage, e_tot=e_tot,
                   delta_e=dE, norm_gorb=g, t=t,
                   gpu=self._gpu_hooks is not None,
                   fp64=self.plan.fp64_phase)
        timings = getattr(self._gpu_hooks, 'timings', None)
        if timings:
            last = timings[-1]
            rec.update(t_jk=last.get('jk'), t_xc=last.get('xc'),
                       t_wait=last.get('wait'))
        self.history.append(rec)
        old = self.plan.stage
        decision = self.plan.after_cycle(dE, g)
        if decision is None:
            return
        if decision[0] == 'fp64':
            self.switches.append(dict(_from=old, to=old, cycle=cycle, t=t,
                                      precision='fp64', forced=decision[1]))
            self._set_gpu(False)
            k_gpu = self.fp64_final_k == 'gpu'
            if self.fp64_final_vv10 == 'gpu' or k_gpu:
                # VV10 stays FP32 on the GPU (or goes back to the CPU); K
                # goes back to the FP64 CPU code, or with fp64_final_k='gpu'
                # runs in the plain FP64 form on the GPU
                kw = dict(self.gpu_kwargs, semilocal=False, k=k_gpu)
                if self.fp64_final_vv10 != 'gpu':
                    kw['vv10'] = False
                if k_gpu:
                    kw['k_precision'] = 'fp64'
                self._gpu_hooks = self._installer(self.mf, **kw)
            self.mf._nsteps_direct = 0
            reset_diis(envs.get('mf_diis'))
            _note(self.mf, 'StagedSCF precision switch FP32 -> FP64 in %s at '
                  'cycle %d (|g|=%.3e, |dE|=%.3e): DIIS reset, full Fock '
                  'rebuild', STAGE_NAMES[old], cycle + 1, g, dE)
            return
        new = decision[1]
        self.switches.append(dict(_from=old, to=new, cycle=cycle, t=t,
                                  forced=decision[2]))
        self.s2_cycles = 0
        self._apply_stage(new)
        reset_diis(envs.get('mf_diis'))
        _note(self.mf, 'StagedSCF switch %s -> %s at cycle %d (|g|=%.3e, '
              '|dE|=%.3e): DIIS reset, full Fock rebuild',
              STAGE_NAMES[old], STAGE_NAMES[new], cycle + 1, g, dE)

    # -- stage settings --------------------------------------------------------
    def _vv10_on(self, stage):
        return (self.vv10_mode != 'nonscf'
                and self.nlc_levels[stage] is not None)

    def _apply_stage(self, stage):
        """Grids of the three operators and the GPU hooks of one stage; the
        next get_veff rebuilds the grids (re-pruned with the current
        density) and, with _nsteps_direct = 0, does a full J/K build."""
        mf, df = self.mf, self.mf.with_df
        mf.grids.level = self.xc_levels[stage]
        if self.nlc_levels[stage] is not None:
            mf.nlcgrids.level = self.nlc_levels[stage]
        mf.nlc = self._saved['nlc'] if self._vv10_on(stage) else 0
        for grids in (mf.grids, mf.nlcgrids):
            if grids.coords is not None:
                grids.reset()
        # pin the SGX grid (turns off SGX's own level_i -> level_f switch)
        level = self.sgx_levels[stage]
        df.grids_level_i = df.grids_level_f = level
        if df.grids is not None:
            df.build(level=level)
        mf._nsteps_direct = 0
        self._set_gpu(stage in self.gpu_stages)

    def _set_gpu(self, on):
        if on and self._gpu_hooks is None:
            self._gpu_hooks = self._installer(self.mf, **self.gpu_kwargs)
        elif not on and self._gpu_hooks is not None:
            self._gpu_hooks.restore_all()
            self._gpu_hooks = None

    # -- reporting ---------------------------------------------------------------
    def info(self):
        """Cycles and wall time per stage, the switches and the history."""
        t_end = time.perf_counter()
        t0 = self._t_attach if self._t_attach is not None else t_end
        stages = {}
        edges = [(s['t'], s['to']) for s in self.switches if 'precision' not in s]
        cur, t_prev = 0, t0
        for t, nxt in edges + [(t_end, None)]:
            entry = stages.setdefault(STAGE_NAMES[cur],
                                      dict(cycles=0, wall=0.0))
            entry['wall'] += t - t_prev
            t_prev = t
            if nxt is not None:
                cur = nxt
        for name, entry in stages.items():
            idx = STAGE_NAMES.index(name)
            entry['cycles'] = sum(1 for h in self.history if h['stage'] == idx)
        return dict(stages=stages, switches=list(self.switches),
                    history=list(self.history), gpu_stages=self.gpu_stages,
                    fp64_final=self.plan.fp64_final,
                    fp64_conv_tol=self.fp64_conv_tol,
                    total_wall=t_end - t0)

    def add_nonscf_vv10(self):
        """vv10_mode='nonscf': one stock FP64 VV10 energy on the final
        density at nlc_production_level, added to mf.e_tot and
        mf.scf_summary['exc'] so that energy_tot() reproduces it.  Returns
        that energy (0.0 in late_scf mode)."""
        if self.vv10_mode != 'nonscf':
            return 0.0
        mf = self.mf
        ni = mf._numint
        grids = mf.nlcgrids
        grids.level = self.nlc_production_level
        if grids.coords is not None:
            grids.reset()
        grids.build(with_non0tab=True)
        xc = mf.xc if ni.libxc.is_nlc(mf.xc) else self._saved['nlc']
        # the class method: a GPU hook on the instance is bypassed
        _, e_nl, _ = type(ni).nr_nlc_vxc(ni, mf.mol, grids, xc,
                                         mf.make_rdm1(),
                                         max_memory=mf.max_memory)
        mf.e_tot += e_nl
        mf.scf_summary['exc'] = mf.scf_summary.get('exc', 0.0) + e_nl
        _note(mf, 'StagedSCF non-SCF VV10 energy = %.10f (grids level %d)',
              e_nl, self.nlc_production_level)
        return e_nl


def _make_mf(mol, xc):
    from pyscf import dft
    return dft.RKS(mol, xc=xc).COSX(pjs=True)


def run_staged(mol, xc='wb97m-v', conv_tol=1e-9, dm0=None, sgx_patch=True,
               staged=None, **staged_kwargs):
    """One staged SCF of an RKS/COSX(pjs=True) mf; returns the info dict
    with e_tot, converged, cycles, nao, xc, the modes, e_nlc, kernel_wall
    and the final density (reference schedule.py:455-485).

    sgx_patch applies the RSH fix of ``core.sgx_patch`` for the run and
    takes it off again afterwards (unless it was already on).  staged_kwargs
    go to StagedSCF; a prepared StagedSCF may be passed as ``staged``.  The
    StagedSCF stays reachable as mf._staged.
    """
    from pyscf_wb97mv_fast_gb300.core import sgx_patch as patch
    mf = _make_mf(mol, xc)
    mf.conv_tol = conv_tol
    patched_here = bool(sgx_patch) and not patch.applied()
    if patched_here:
        patch.apply()
    try:
        if staged is None:
            staged = StagedSCF(mf, **staged_kwargs)
        with staged:
            t0 = time.perf_counter()
            mf.kernel(dm0=dm0)
            e_nl = staged.add_nonscf_vv10()
            wall = time.perf_counter() - t0
        info = staged.info()
        info.update(e_tot=float(mf.e_tot), converged=bool(mf.converged),
                    cycles=int(mf.cycles), nao=int(mol.nao), xc=xc,
                    vv10_mode=staged.vv10_mode, s2_mode=staged.s2_mode,
                    e_nlc=float(e_nl), kernel_wall=wall, dm=mf.make_rdm1())
        mf._staged = staged
        return info
    finally:
        if patched_here:
            patch.revert()
