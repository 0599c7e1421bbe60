"""GpuKBuilder.get_k's host logic on the CPU (reference gpu/sgx_k.py:663-751):
the projector and its symmetric form, the symmetrisation, the second omega
of a multi-omega build handed out from the pending set, the grid-state
cache, and the phase timing of PYSCF_WB97MV_KPROFILE=1.  The engine is a
stand-in on the CPU device that returns K_j = s_j * QD with s_j = (1 +
omega_j) * sum(w): what get_k does with it is the subject."""
import types

import numpy as np
import pytest
import torch

from pyscf_wb97mv_fast_gb300.gpu.sgx_k import (GpuKBuilder, SyntheticSGX,
                                               get_k_only_gpu)

NAO = 5


class FakeEngine:
    def __init__(self):
        self.nao = NAO
        self.device = torch.device('cpu')
        self.calls = []
        self.last_stats = {}

    def relative(self, coords):
        return torch.as_tensor(coords, dtype=torch.float64).contiguous()

    def _k(self, w, qd, omegas):
        s = float(w.sum())
        return torch.stack([(1.0 + om) * s * qd for om in omegas])

    def get_k_multi(self, c, w, qd, omegas, tile_tol=1e-11, tile_pts=0,
                    gemm='ozaki', profile=False):
        self.calls.append(('multi', tuple(omegas), profile))
        self.last_stats = {'pairs_kept': 1, 'phase_ms': {'g': 1.0}}
        return self._k(w, qd, omegas)

    def get_k(self, c, w, qd, omega, tile_tol=1e-11, tile_pts=0, gemm='ozaki',
              profile=False):
        self.calls.append(('single', omega, profile))
        self.last_stats = {'pairs_kept': 1}
        return self._k(w, qd, (omega,))[0]


def _builder(omegas=(0.0, 0.3)):
    b = GpuKBuilder(types.SimpleNamespace(nao=NAO), omegas=omegas)
    b.engine = FakeEngine()
    b.nao = NAO
    b.mem_budget = 1 << 30
    b._built = True
    return b


def _sgx(proj=None, sym=False, npts=7):
    grids = types.SimpleNamespace(coords=np.zeros((npts, 3)),
                                  weights=np.full(npts, 0.5))
    mol = types.SimpleNamespace(nao=NAO, omega=0.0)
    return SyntheticSGX(mol, grids, proj=proj, sym=sym)


def _dm(seed):
    c = np.random.default_rng(seed).normal(size=(NAO, 2))
    return c @ c.T


def _expect(dm, proj, sym, omega, wsum):
    qd = proj @ dm
    K = (1.0 + omega) * wsum * qd
    if sym:
        K = proj.T @ K
    return 0.5 * (K + K.T)


@pytest.mark.parametrize('sym', [False, True])
def test_projector_symmetrisation_and_pending_second_omega(sym):
    b = _builder()
    proj = np.eye(NAO) + 0.1 * np.random.default_rng(1).normal(size=(NAO, NAO))
    sgx = _sgx(proj, sym)
    dm = _dm(0)
    K0 = get_k_only_gpu(b, sgx, dm)
    assert np.allclose(K0, _expect(dm, proj, sym, 0.0, 3.5), atol=1e-13)
    assert np.array_equal(K0, K0.T)
    sgx.mol.omega = 0.3
    K3 = get_k_only_gpu(b, sgx, dm)
    assert b.last_stats['from_multi']
    assert np.allclose(K3, _expect(dm, proj, sym, 0.3, 3.5), atol=1e-13)
    assert b.engine.calls == [('multi', (0.0, 0.3), False)]
    # another density: built afresh, and the pending set is dropped
    get_k_only_gpu(b, sgx, _dm(1))
    sgx.mol.omega = 0.0
    get_k_only_gpu(b, sgx, dm)
    assert len(b.engine.calls) == 3 and not b.last_stats['from_multi']


def test_one_build_per_call_without_omegas_and_grid_cache():
    b = _builder(omegas=None)
    sgx = _sgx()
    dm = _dm(2)
    for _ in range(2):
        get_k_only_gpu(b, sgx, dm)
    assert [c[0] for c in b.engine.calls] == ['single', 'single']
    assert len(b._grids_states) == 1
    for n in range(8, 14):                     # at most four grid states kept
        get_k_only_gpu(b, _sgx(npts=n), dm)
    assert len(b._grids_states) == 4


def test_phase_timing_switch(monkeypatch):
    b = _builder()
    sgx = _sgx()
    get_k_only_gpu(b, sgx, _dm(3))
    assert 'phases' not in b.last_stats and b.engine.calls[-1][2] is False
    monkeypatch.setenv('PYSCF_WB97MV_KPROFILE', '1')
    get_k_only_gpu(b, sgx, _dm(4))
    ph = b.last_stats['phases']
    assert list(ph) == ['checks', 'build', 'pjs', 'grid_state', 'proj_dm',
                        'kernel', 'post', 'to_host']
    assert min(ph.values()) >= 0.0 and b.engine.calls[-1][2] is True
    assert b.last_stats['phase_ms'] == {'g': 1.0}


def test_inputs_outside_the_contract_raise():
    from pyscf_wb97mv_fast_gb300 import _native
    b = _builder()
    sgx = _sgx()
    with pytest.raises(_native.Unsupported):
        get_k_only_gpu(b, sgx, _dm(5), hermi=0)
    with pytest.raises(_native.Unsupported):
        b.get_k(sgx, np.zeros((NAO, NAO + 1)), 0.0)
    asym = _dm(6)
    asym[0, 1] += 1.0
    with pytest.raises(_native.Unsupported):
        b.get_k(sgx, asym, 0.0)
    with pytest.raises(_native.Unsupported):
        b.get_k(sgx, np.eye(NAO + 1), 0.0)
    assert b.engine.calls == []
