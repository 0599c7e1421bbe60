"""The K hook of install_gpu on the CPU (the reference's integration cases,
tests/gpu/test_install.py:288-410): this mf's full-range SGX object and a
long-range copy created after install both reach one builder, built once;
the second omega of an SCF cycle comes from the multi-omega build; a grid
rebuild is picked up; other SGX objects keep the original; k_stats gets
one record per call.  The builder's engine is a stand-in on the CPU device
(K_j = (1 + omega_j) * sum(w) * QD), so no GPU is needed."""
import types

import numpy as np
import pytest
import torch

from pyscf_wb97mv_fast_gb300.basis import Molecule
from pyscf_wb97mv_fast_gb300.gpu import sgx_k
from pyscf_wb97mv_fast_gb300.gpu.install import install_gpu
from pyscf_wb97mv_fast_gb300.gpu.sgx_k import SyntheticSGX
from pyscf_wb97mv_fast_gb300.systems import water_dimer


class FakeEngine:
    def __init__(self, nao):
        self.nao = nao
        self.device = torch.device('cpu')
        self.calls = []
        self.last_stats = {}

    def relative(self, coords):
        return torch.as_tensor(coords, dtype=torch.float64).contiguous()

    def get_k_multi(self, c, w, qd, omegas, **kw):
        self.calls.append(tuple(omegas))
        self.last_stats = {'pairs_kept': 1}
        return torch.stack([(1.0 + om) * float(w.sum()) * qd for om in omegas])


@pytest.fixture
def setup(monkeypatch):
    mol = Molecule.build(water_dimer(), 'synthetic-svp')
    builds = []

    def fake_build(self):
        if self._built:
            return
        builds.append(self)
        self.engine = FakeEngine(mol.nao)
        self.nao = mol.nao
        self.mem_budget = 1 << 30
        self._built = True

    monkeypatch.setattr(sgx_k.GpuKBuilder, '_build', fake_build)
    monkeypatch.setattr(torch.cuda, 'mem_get_info', lambda dev=None: (1 << 34, 1 << 35))

    def grids(n, w):
        return types.SimpleNamespace(coords=np.zeros((n, 3)), weights=np.full(n, w))

    full = SyntheticSGX(types.SimpleNamespace(nao=mol.nao, omega=0.0), grids(9, 1.0))
    full._rsh_df = {}
    mf = types.SimpleNamespace(mol=mol, with_df=full, _numint=types.SimpleNamespace())
    mod = types.ModuleType('fake_sgx_jk')
    mod.get_k_only = lambda sgx, dm, hermi=1, tol=1e-13: 'original'
    hooks = install_gpu(mf, k=True, semilocal=False, vv10=False, overlap=False,
                        sgx_jk_module=mod, k_omegas=(0.0, 0.3))
    yield mol, mf, mod, hooks, builds, grids
    hooks.restore_all()


def _dm(nao, seed):
    c = np.random.default_rng(seed).normal(size=(nao, 4))
    return c @ c.T


def test_full_and_lazily_added_long_range_copy_share_one_build(setup):
    mol, mf, mod, hooks, builds, grids = setup
    full = mf.with_df
    dm = _dm(mol.nao, 0)
    K0 = mod.get_k_only(full, dm)
    # the long-range copy appears after install, as PySCF creates it lazily
    lr = SyntheticSGX(types.SimpleNamespace(nao=mol.nao, omega=0.3), full.grids)
    full._rsh_df['0.3'] = lr
    K3 = mod.get_k_only(lr, dm)
    assert np.allclose(K0, 9.0 * dm, atol=1e-12)
    assert np.allclose(K3, 1.3 * 9.0 * dm, atol=1e-12)
    (b,) = builds                                # built once
    assert b.engine.calls == [(0.0, 0.3)]        # one multi-omega build
    assert len(hooks.k_stats) == 2 and hooks.k_stats[1]['from_multi']
    other = SyntheticSGX(types.SimpleNamespace(nao=mol.nao, omega=0.0), full.grids)
    assert mod.get_k_only(other, dm) == 'original'
    assert len(hooks.k_stats) == 2


def test_grid_rebuild_is_picked_up(setup):
    mol, mf, mod, hooks, builds, grids = setup
    dm = _dm(mol.nao, 1)
    K = mod.get_k_only(mf.with_df, dm)
    assert np.allclose(K, 9.0 * dm, atol=1e-12)
    mf.with_df.grids = grids(12, 0.5)            # a new grids object
    mf.with_df._pjs_data = None
    K = mod.get_k_only(mf.with_df, dm)
    assert np.allclose(K, 6.0 * dm, atol=1e-12)
    assert len(builds) == 1 and len(builds[0].engine.calls) == 2
