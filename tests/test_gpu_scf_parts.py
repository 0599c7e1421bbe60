"""The SCF's device pieces against the oracle: one-electron integrals
(wb_scf_int1e) and the Hartree potential on grid points (wb_hartree)."""
import numpy as np
import pytest

import oracle
from helpers import density, dimer, waters

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize('basis,gen', [('synthetic-svp', False),
                                       ('synthetic-tzvp', False),
                                       ('synthetic-svp', True)])
def test_int1e_matches_oracle(basis, gen):
    from pyscf_wb97mv_fast_gb300.cosx import CosxEngine
    mol = dimer(basis, gen)
    eng = CosxEngine(mol, device=0)
    S, T, V = (x.cpu().numpy() for x in eng.int1e())
    So, To, Vo = oracle.int1e(mol)
    for got, ref in ((S, So), (T, To), (V, Vo)):
        assert np.abs(got - ref).max() < 1e-12 * np.abs(ref).max()
        np.testing.assert_array_equal(got, got.T)


def _points(mol, n, seed):
    from pyscf_wb97mv_fast_gb300.grids import build_grids
    g = build_grids(mol, level=0)
    idx = np.sort(np.random.default_rng(seed).choice(g.size, n, replace=False))
    return g.coords[idx]


@pytest.mark.parametrize('basis', ['synthetic-svp', 'synthetic-tzvp'])
def test_hartree_matches_oracle(basis):
    import torch
    from pyscf_wb97mv_fast_gb300.cosx import CosxEngine
    mol = dimer(basis)
    eng = CosxEngine(mol, device=0)
    pts = _points(mol, 700, 1)
    dm = density(mol.nao, 10, seed=2)
    ref = oracle.hartree(mol, pts, dm)
    c = eng.relative(pts)
    d = torch.as_tensor(dm, device='cuda')
    v64 = eng.hartree(c, d, tol=0.0, fp64=True).cpu().numpy()
    assert np.abs(v64 - ref).max() < 1e-12 * np.abs(ref).max()
    v32 = eng.hartree(c, d, tol=0.0, fp64=False).cpu().numpy()
    assert np.abs(v32 - ref).max() < 2e-6 * np.abs(ref).max()
    # screened: the locked bound times |D| per pair keeps the error below
    # tol per kept-out pair
    vs = eng.hartree(c, d, tol=1e-11, fp64=True, stats=True).cpu().numpy()
    assert np.abs(vs - ref).max() < 1e-11 * eng.npairs
    # bitwise reproducible
    np.testing.assert_array_equal(eng.hartree(c, d, tol=0.0, fp64=False).cpu().numpy(),
                                  v32)


def test_hartree_on_a_cluster_screens_and_matches():
    import torch
    from pyscf_wb97mv_fast_gb300.cosx import CosxEngine
    mol = waters(6, box=8.0, seed=4)
    eng = CosxEngine(mol, device=0)
    pts = _points(mol, 1500, 3)
    dm = density(mol.nao, 30, seed=5)
    ref = oracle.hartree(mol, pts, dm)
    d = torch.as_tensor(dm, device='cuda')
    v = eng.hartree(eng.relative(pts), d, tol=1e-11, fp64=True, stats=True).cpu().numpy()
    kept = eng.last_hartree_kept
    assert 0 < kept < (-(-len(pts) // 32)) * eng.npairs
    assert np.abs(v - ref).max() < 1e-11 * eng.npairs
