"""Semilocal XC flow on the GPU (gpu_nr_rks) against the FP64 oracle flow
(reference tests: tests/gpu/test_xc_vv10.py:66-86 -- there against PySCF's
nr_rks: nelec relative 1e-6, |dE| 1e-5, vmat 1e-5 for the FP32 flow).

The GPU flow rounds two intermediates to FP32 (T = D^T X and the Fock-side
planes) and keeps everything else FP64-accurate, so beside the reference's
gates it is held to 1e-6 relative errors."""
import types

import numpy as np
import pytest

import oracle
from helpers import ToyFunctional, ToyNumInt, density, dimer, grid_subset, waters

pytestmark = pytest.mark.gpu


def _flow(mol, coords, weights, dm, xctype, tile_pts=None):
    from pyscf_wb97mv_fast_gb300.gpu.xc import XcContext, gpu_nr_rks
    ctx = XcContext(mol, functional_factory=lambda xc, ni: ToyFunctional(xctype))
    if tile_pts:
        ctx.tile_pts = tile_pts
    grids = types.SimpleNamespace(coords=coords, weights=weights)
    return gpu_nr_rks(ctx, ToyNumInt(xctype), mol, grids, 'toy', dm)


@pytest.mark.parametrize('xctype', ['LDA', 'GGA', 'MGGA'])
def test_nr_rks_matches_oracle_flow(xctype):
    mol = dimer()
    coords, weights = grid_subset(mol, 1, 6000, 4)
    dm = density(mol.nao, 5, 2)
    n, e, v = _flow(mol, coords, weights, dm, xctype)
    n0, e0, v0 = oracle.nr_rks(mol, coords, weights, dm, ToyFunctional(xctype), xctype)
    # the reference's FP32-flow gates
    assert abs(n - n0) / n0 < 1e-6
    assert abs(e - e0) < 1e-5
    assert np.max(np.abs(v - v0)) < 1e-5
    # and relative 1e-6
    assert abs(e - e0) <= 1e-6 * abs(e0), (e, e0)
    assert np.max(np.abs(v - v0)) <= 1e-6 * np.abs(v0).max()
    assert np.array_equal(v, v.T)


def test_nr_rks_drug_like_tzvp():
    """Heavier elements and f shells (a seeded drug-like molecule)."""
    from pyscf_wb97mv_fast_gb300.basis import Molecule
    from pyscf_wb97mv_fast_gb300.systems import drug_like
    mol = Molecule.build(drug_like(2), 'synthetic-tzvp')
    coords, weights = grid_subset(mol, 1, 4000, 9)
    dm = density(mol.nao, 30, 4)
    n, e, v = _flow(mol, coords, weights, dm, 'MGGA')
    n0, e0, v0 = oracle.nr_rks(mol, coords, weights, dm, ToyFunctional('MGGA'), 'MGGA')
    assert abs(n - n0) / n0 < 1e-6
    assert abs(e - e0) <= 1e-6 * abs(e0)
    assert np.max(np.abs(v - v0)) <= 1e-6 * np.abs(v0).max()


def test_tiles_give_the_one_tile_result():
    """Several tiles (a ragged last one) sum to the one-tile result up to
    the order of the FP64 sums."""
    mol = dimer()
    coords, weights = grid_subset(mol, 1, 5000, 6)
    dm = density(mol.nao, 5, 3)
    n1, e1, v1 = _flow(mol, coords, weights, dm, 'MGGA')
    n2, e2, v2 = _flow(mol, coords, weights, dm, 'MGGA', tile_pts=1536)
    assert abs(n1 - n2) <= 1e-12 * abs(n1)
    assert abs(e1 - e2) <= 1e-11 * abs(e1)
    assert np.max(np.abs(v1 - v2)) <= 1e-10 * np.abs(v1).max()


def test_potential_is_the_energy_derivative_at_scale():
    """Size-independent check on a 6-water cluster with its full level-0
    grid: tr(vmat P) = d E_xc(D + h P) / dh (central difference), to the
    FP32 rounding of the flow."""
    from pyscf_wb97mv_fast_gb300.grids import build_grids
    mol = waters(6, 7.0, 5)
    g = build_grids(mol, level=0)
    dm = density(mol.nao, 30, 7)
    rng = np.random.default_rng(8)
    P = rng.normal(size=dm.shape)
    P = 0.5 * (P + P.T) / np.abs(P).max()
    _, _, v = _flow(mol, g.coords, g.weights, dm, 'MGGA')
    h = 1e-3
    ep = _flow(mol, g.coords, g.weights, dm + h * P, 'MGGA')[1]
    em = _flow(mol, g.coords, g.weights, dm - h * P, 'MGGA')[1]
    fd = (ep - em) / (2 * h)
    an = float(np.sum(v * P))
    # FP32 rounding noise of E over 2h (~1e-4 relative) bounds the match;
    # a wrong factor anywhere in the chain rule or the Fock assembly is O(1)
    assert abs(fd - an) <= 1e-3 * max(1.0, abs(an)), (fd, an)
