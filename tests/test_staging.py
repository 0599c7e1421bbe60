"""Staged SCF driver and the SGX RSH patch, on CPU with a stand-in mf.

The stand-in follows the parts of PySCF's SCF loop the driver relies on
(scf/hf.py kernel): per cycle a get_veff (here: a snapshot of the settings
it would read), the energy and orbital-gradient norm, then
``check_convergence`` (when callable) before ``callback``; after a converged
loop with conv_check on, one extra cycle whose convergence test sees the
same cycle number.  Energies depend on the settings in force, so a missed
or early switch shows up as a different history.  Reference tests:
tests/staging (StagedSCF switching, restore) of pyscf_wb97mv_fast.
"""
import math
from contextlib import contextmanager

import numpy as np
import pytest

from pyscf_wb97mv_fast_gb300.core import sgx_patch
from pyscf_wb97mv_fast_gb300.staging import schedule
from pyscf_wb97mv_fast_gb300.staging.schedule import StagePlan, StagedSCF


class Grids:
    def __init__(self, level):
        self.level = level
        self.coords = None
        self.resets = 0
        self.built = []

    def reset(self):
        self.coords = None
        self.resets += 1

    def build(self, with_non0tab=False):
        self.coords = np.zeros((4, 3))
        self.built.append(self.level)


class SGX:
    def __init__(self):
        self.grids_level_i, self.grids_level_f = 0, 2
        self.grids = None
        self.built = []

    def build(self, level=None):
        self.grids = ('sgx', level)
        self.built.append(level)


class DIIS:
    def __init__(self):
        self.resets = 0
        self._H = 'history'

    def __setattr__(self, name, value):
        if name == '_H' and value is None:
            object.__setattr__(self, 'resets', self.resets + 1)
        object.__setattr__(self, name, value)


class Libxc:
    @staticmethod
    def is_nlc(xc):
        return xc.lower() == 'wb97m-v'


class NumInt:
    libxc = Libxc()
    calls = []

    def nr_nlc_vxc(self, mol, grids, xc, dm, max_memory=2000):
        NumInt.calls.append((grids.level, xc))
        return 10.0, -0.0123, np.zeros((2, 2))


class Hooks:
    def __init__(self, mf, kw):
        self.mf, self.kw = mf, kw
        mf.gpu = kw
        self.timings = []

    def restore_all(self):
        self.mf.gpu = None


class FakeMF:
    """RKS/COSX stand-in with a convergent model SCF."""
    callback = None               # class attributes, as on PySCF's SCF
    check_convergence = None

    def __init__(self, decay=0.2, max_cycle=60):
        self.with_df = SGX()
        self.grids = Grids(3)
        self.nlcgrids = Grids(1)
        self.nlc = ''
        self.xc = 'wb97m-v'
        self.conv_check = True
        self.conv_tol = 1e-9
        self.conv_tol_grad = None
        self.max_memory = 4000
        self.mol = 'mol'
        self._numint = NumInt()
        self._nsteps_direct = 7
        self.scf_summary = {}
        self.gpu = None
        self.decay = decay
        self.max_cycle = max_cycle
        self.diis = DIIS()
        self.veff_log = []

    def make_rdm1(self):
        return np.eye(2)

    def _get_veff(self):
        """What a get_veff sees; (re)builds grids like initialize_grids."""
        for g in (self.grids, self.nlcgrids):
            if g.coords is None:
                g.build(with_non0tab=True)
        if self.with_df.grids is None:        # SGX builds on first use
            self.with_df.build(level=self.with_df.grids_level_i)
        snap = dict(xc=self.grids.level, nlc=self.nlc,
                    nlc_level=self.nlcgrids.level,
                    sgx=(self.with_df.grids_level_i, self.with_df.grids_level_f),
                    full=self._nsteps_direct == 0,
                    gpu=None if self.gpu is None else dict(self.gpu))
        self._nsteps_direct += 1
        self.veff_log.append(snap)
        return snap

    def _energy(self, snap, g):
        base = -76.0 - 1e-4 * snap['xc'] - 2e-5 * snap['sgx'][0]
        if snap['nlc'] != 0:
            base -= 1e-5 * snap['nlc_level']
        if snap['gpu'] is not None:
            base += 3e-8          # FP32 offset of the GPU flows
        return base + 0.5 * g * g

    def kernel(self, dm0=None):
        g, e_last, conv, cycle = 0.5, 0.0, False, 0
        key = None
        for cycle in range(self.max_cycle):
            snap = self._get_veff()
            k = (snap['xc'], snap['nlc'], snap['nlc_level'], snap['sgx'],
                 snap['gpu'] is None)
            if key is not None and k != key:
                g = max(g, 5e-5)          # a switch disturbs the density
            key = k
            g *= self.decay
            e_tot = self._energy(snap, g)
            envs = dict(cycle=cycle, e_tot=e_tot, last_hf_e=e_last,
                        norm_gorb=g, mf_diis=self.diis)
            if callable(self.check_convergence):
                conv = self.check_convergence(envs)
            else:
                conv = (abs(e_tot - e_last) < self.conv_tol
                        and g < math.sqrt(self.conv_tol))
            if callable(self.callback):
                self.callback(envs)
            e_last = e_tot
            if conv:
                break
        if conv and self.conv_check:
            snap = self._get_veff()
            g *= self.decay
            e_tot = self._energy(snap, g)
            envs = dict(cycle=cycle, e_tot=e_tot, last_hf_e=e_last,
                        norm_gorb=g, mf_diis=self.diis)
            if callable(self.check_convergence):
                conv = self.check_convergence(envs)
            if callable(self.callback):
                self.callback(envs)
        self.converged, self.cycles, self.e_tot = conv, cycle + 1, e_tot
        return e_tot


def installer(calls):
    def install(mf, **kw):
        calls.append(dict(kw))
        return Hooks(mf, kw)
    return install


# -- StagePlan --------------------------------------------------------------
def test_plan_switches_in_order():
    p = StagePlan()
    assert p.after_cycle(1.0, 2e-3) is None
    assert p.after_cycle(1.0, 5e-4) == ('stage', 1, False)
    assert p.after_cycle(1e-5, 1e-4) is None
    assert p.after_cycle(5e-7, 1e-4) == ('stage', 2, False)
    assert p.after_cycle(1e-12, 1e-9) is None          # no FP64 tail
    assert p.stage == 2 and p.may_converge


def test_plan_forced_switches_and_gates():
    p = StagePlan(max_s1_cycles=3, tau2_g=1e-3)
    p.after_cycle(1.0, 1e-4)
    assert p.stage == 1
    assert p.after_cycle(1e-9, 5e-3) is None          # |g| gate holds S1
    assert p.after_cycle(1e-9, 5e-3) is None
    assert p.after_cycle(1e-9, 5e-3) == ('stage', 2, True)

    q = StagePlan(fp64_final=True, max_fp32_s2_cycles=2, tau_fp64_g=1e-6)
    q.after_cycle(1.0, 1e-4)
    q.after_cycle(1e-7, 1e-4)
    assert q.stage == 2 and not q.may_converge
    assert q.after_cycle(1e-9, 1e-4) is None          # |g| above tau_fp64_g
    assert q.after_cycle(1e-9, 1e-4) == ('fp64', True)
    assert q.fp64_phase and q.may_converge
    assert q.after_cycle(1e-9, 1e-9) is None          # one switch only

    r = StagePlan(fp64_final=True, tau_fp64=1e-7)
    r.after_cycle(1.0, 1e-4)
    r.after_cycle(1e-7, 1e-4)
    assert r.after_cycle(5e-8, 1e-5) == ('fp64', False)


# -- StagedSCF on the stand-in ---------------------------------------------------
def test_argument_checks():
    mf = FakeMF()
    with pytest.raises(TypeError):
        StagedSCF(object())
    for kw in (dict(gpu_stages=(3,)), dict(fp64_final=True),
               dict(fp64_final_vv10='x'), dict(fp64_conv_tol=1e-8),
               dict(vv10_mode='x'), dict(s2_mode='x'),
               dict(xc_levels=(1, 2))):
        with pytest.raises(ValueError):
            StagedSCF(mf, **kw)
    s = StagedSCF(mf).attach()
    with pytest.raises(RuntimeError):
        s.attach()
    s.restore()


def test_cpu_run_walks_the_three_stages_and_restores():
    mf = FakeMF()
    user = []
    mf.callback = lambda envs: user.append(envs['cycle'])
    calls = []
    with StagedSCF(mf, installer=installer(calls)) as st:
        mf.kernel()
        info = st.info()
    assert calls == []
    assert [s['to'] for s in st.switches] == [1, 2]
    assert mf.converged
    # settings seen by get_veff, per stage
    seen = {}
    for h, snap in zip(st.history, mf.veff_log):
        seen.setdefault(h['stage'], set()).add(
            (snap['xc'], snap['nlc'], snap['nlc_level'], snap['sgx']))
    assert seen[0] == {(1, 0, 1, (1, 1))}
    assert seen[1] == {(3, '', 1, (1, 1))}
    assert seen[2] == {(3, '', 3, (2, 2))}
    # a full Fock build right after every switch, DIIS dropped at each
    first = [i for i in range(1, len(st.history))
             if st.history[i]['stage'] != st.history[i - 1]['stage']]
    assert all(mf.veff_log[i]['full'] for i in first)
    assert mf.diis.resets == 2
    assert mf.with_df.built == [1, 1, 2]
    assert info['stages']['S2']['cycles'] >= 1
    assert sum(v['cycles'] for v in info['stages'].values()) == len(st.history)
    # user callback kept, everything restored
    assert len(user) == len(st.history)
    assert mf.nlc == '' and mf.conv_check is True
    assert (mf.grids.level, mf.nlcgrids.level) == (3, 1)
    assert (mf.with_df.grids_level_i, mf.with_df.grids_level_f) == (0, 2)
    assert callable(mf.callback) and mf.check_convergence is None
    mf.callback(dict(cycle=-5))
    assert user[-1] == -5


def test_gpu_stages_with_fp64_tail():
    mf = FakeMF()
    calls = []
    st = StagedSCF(mf, gpu_stages=(0, 1, 2), fp64_final=True,
                   gpu_kwargs=dict(k=True, k_tile_tol=1e-11),
                   installer=installer(calls))
    with st:
        mf.kernel()
    # one install for S0..S2 (kept across switches), then VV10 only for
    # the FP64 tail
    assert calls[0] == dict(k=True, k_tile_tol=1e-11)
    assert calls[1] == dict(k=False, k_tile_tol=1e-11, semilocal=False)
    assert len(calls) == 2
    prec = [s for s in st.switches if s.get('precision') == 'fp64']
    assert len(prec) == 1 and not prec[0]['forced']
    i = next(i for i, h in enumerate(st.history) if h['fp64'])
    # convergence only after the switch, on FP64 cycles
    assert all(not h['fp64'] for h in st.history[:i])
    assert st.history[-1]['fp64'] and mf.converged
    assert mf.veff_log[i]['full'] and mf.veff_log[i]['gpu']['k'] is False
    assert mf.gpu is None          # hooks off after restore


@pytest.mark.parametrize('vv10', ['gpu', 'cpu'])
def test_fp64_tail_on_the_gpu(vv10):
    """fp64_final_k='gpu' (an addition): the FP64 tail keeps K on the GPU in
    its plain FP64 form; VV10 stays on the GPU only with
    fp64_final_vv10='gpu'."""
    mf = FakeMF()
    calls = []
    st = StagedSCF(mf, gpu_stages=(0, 1, 2), fp64_final=True, fp64_final_k='gpu',
                   fp64_final_vv10=vv10, gpu_kwargs=dict(k=True, k_tile_tol=1e-11),
                   installer=installer(calls))
    with st:
        mf.kernel()
    tail = dict(k=True, k_tile_tol=1e-11, semilocal=False, k_precision='fp64')
    if vv10 == 'cpu':
        tail['vv10'] = False
    assert calls == [dict(k=True, k_tile_tol=1e-11), tail]
    i = next(i for i, h in enumerate(st.history) if h['fp64'])
    assert mf.veff_log[i]['full'] and mf.veff_log[i]['gpu']['k'] is True
    assert st.history[-1]['fp64'] and mf.converged
    assert mf.gpu is None
    with pytest.raises(ValueError):
        StagedSCF(FakeMF(), fp64_final=True, fp64_final_k='x')


def test_fp64_conv_tol_and_steps_mode_turn_conv_check_off():
    mf = FakeMF()
    seen = []
    mf.callback = None
    st = StagedSCF(mf, s2_mode='steps', s2_steps=2)
    with st:
        seen.append(mf.conv_check)
        mf.kernel()
    assert seen == [False] and mf.conv_check is True
    s2 = [h for h in st.history if h['stage'] == 2]
    assert len(s2) == 2 and mf.converged

    mf2 = FakeMF()
    st2 = StagedSCF(mf2, gpu_stages=(2,), fp64_final=True,
                    fp64_conv_tol=1e-7, installer=installer([]))
    with st2:
        assert mf2.conv_check is False
        mf2.kernel()
    last = st2.history[-1]
    assert last['fp64'] and last['delta_e'] < 1e-7


def test_user_check_convergence_and_extra_cycle():
    mf = FakeMF()
    asked = []

    def user_check(envs):
        asked.append(envs['cycle'])
        return envs['norm_gorb'] < 1e-7
    mf.check_convergence = user_check
    with StagedSCF(mf) as st:
        mf.kernel()
    assert asked and mf.converged
    assert mf.check_convergence is user_check
    # stock test with the extra conv_check cycle: the repeated cycle number
    # gets the relaxed thresholds
    mf2 = FakeMF()
    st2 = StagedSCF(mf2).attach()
    check = mf2.check_convergence
    st2.plan.stage = 2
    env = dict(cycle=4, e_tot=-1.0, last_hf_e=-1.0 - 5e-9, norm_gorb=1e-4)
    assert check(env) is False
    assert check(dict(env)) is True       # same cycle: |dE| < 10 conv_tol
    st2.restore()


def test_nonscf_vv10():
    mf = FakeMF()
    NumInt.calls.clear()
    mf.e_tot = -76.0
    st = StagedSCF(mf, vv10_mode='nonscf')
    with st:
        mf.kernel()
        assert all(s['nlc'] == 0 for s in mf.veff_log)
        e0 = mf.e_tot
        mf._numint.nr_nlc_vxc = lambda *a, **k: (_ for _ in ()).throw(
            AssertionError('instance hook must be bypassed'))
        e_nl = st.add_nonscf_vv10()
    assert e_nl == -0.0123
    assert mf.e_tot == pytest.approx(e0 - 0.0123, abs=1e-15)
    assert mf.scf_summary['exc'] == -0.0123
    assert NumInt.calls == [(3, 'wb97m-v')]
    assert StagedSCF(FakeMF()).add_nonscf_vv10() == 0.0


def test_run_staged_with_a_stand_in(monkeypatch):
    made = []

    def make(mol, xc):
        mf = FakeMF()
        mf.mol = mol
        made.append(mf)
        return mf

    class Mol:
        nao = 24
    monkeypatch.setattr(schedule, '_make_mf', make)
    info = schedule.run_staged(Mol(), conv_tol=1e-10, sgx_patch=False,
                               tau1=1e-3)
    mf = made[0]
    assert mf.conv_tol == 1e-10 and mf._staged is not None
    assert info['converged'] and info['nao'] == 24
    assert info['cycles'] == mf.cycles and info['e_tot'] == mf.e_tot
    assert info['e_nlc'] == 0.0 and info['dm'].shape == (2, 2)
    assert set(info['stages']) == {'S0', 'S1', 'S2'}


# -- SGX RSH patch ---------------------------------------------------------------
def _fake_sgx_module():
    log = []

    class Mol:
        omega = 0.0

        @contextmanager
        def with_range_coulomb(self, omega):
            old, self.omega = self.omega, omega
            try:
                yield self
            finally:
                self.omega = old

    class SGX:
        def __init__(self):
            self.mol = Mol()
            self._rsh_df = {}
            self._vjopt = 'vj'
            self._overlap_correction_matrix = 'q'
            self._pjs_data = 'full-range bounds'

        def copy(self):
            new = SGX.__new__(SGX)
            new.__dict__.update(self.__dict__)
            return new

        def get_jk(self, dm, hermi=1, vhfopt=None, with_j=True, with_k=True,
                   direct_scf_tol=1e-13, omega=None):
            log.append((self, vhfopt, with_j, with_k, direct_scf_tol,
                        self.mol.omega, self._pjs_data))
            return 'jk'

    class Module:
        pass
    mod = Module()
    mod.SGX = SGX
    return mod, log


def test_sgx_patch_routes_the_rsh_branch():
    mod, log = _fake_sgx_module()
    stock = mod.SGX.get_jk
    sgx_patch.apply(mod)
    sgx_patch.apply(mod)                      # idempotent
    assert sgx_patch.applied()
    try:
        s = mod.SGX()
        assert s.get_jk('dm', 1, None, False, True, 1e-11) == 'jk'
        assert log[-1][0] is s and log[-1][2:5] == (False, True, 1e-11)
        s.get_jk('dm', 1, None, False, True, 1e-11, omega=0.3)
        rsh = s._rsh_df['0.300000']
        who, vhfopt, wj, wk, tol, om, pjs = log[-1]
        assert who is rsh and (vhfopt, wj, wk, tol) == (None, False, True, 1e-11)
        assert om == 0.3 and pjs is None          # attenuated, own bounds
        assert rsh._rsh_df is None and rsh._vjopt is None
        assert rsh._overlap_correction_matrix is None
        assert s._pjs_data == 'full-range bounds' and s.mol.omega == 0.0
        s.get_jk('dm', omega=0.3)
        assert log[-1][0] is rsh and len(s._rsh_df) == 1
    finally:
        sgx_patch.revert()
    assert mod.SGX.get_jk is stock and not sgx_patch.applied()
    sgx_patch.revert()                        # no-op
