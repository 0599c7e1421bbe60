"""The plain FP64 form of the K build (wb_cosx_get_k_fp64) against the FP64
oracle and against the mixed-precision path.  It is the comparison point of
the mixed-precision path: same steps, same screen, everything in FP64.  All
calls go through the C ABI."""
import numpy as np
import pytest

import oracle
from helpers import density, dimer, grid_subset, local_density, waters

pytestmark = pytest.mark.gpu


def _torch():
    import torch
    return torch


def _k64(mol, coords, weights, dm, omegas, tile_tol=0.0, eng=None):
    torch = _torch()
    from pyscf_wb97mv_fast_gb300.cosx import CosxEngine
    eng = eng or CosxEngine(mol)
    c = eng.relative(coords)
    w = torch.as_tensor(weights, device=eng.device)
    qd = torch.as_tensor(dm, device=eng.device)
    K = eng.get_k_fp64(c, w, qd, omegas, tile_tol=tile_tol)
    K = ((K + K.transpose(1, 2)) * 0.5).cpu().numpy()
    return K, eng.last_stats


@pytest.mark.parametrize('basis,gen', [('synthetic-svp', False),
                                       ('synthetic-tzvp', False),
                                       ('synthetic-svp', True)])
def test_fp64_k_matches_oracle(basis, gen):
    """FP64 all the way: agreement with the FP64 oracle at FP64 rounding
    level (1e-11 relative; the mixed-precision gate is 1e-6)."""
    mol = dimer(basis, gen)
    coords, weights = grid_subset(mol, 1, 3000, 1)
    dm = density(mol.nao, 10, 2)
    K, st = _k64(mol, coords, weights, dm, (0.0, 0.3))
    assert st['pairs_kept'] == st['pairs_total']
    for j, om in enumerate((0.0, 0.3)):
        Kref = oracle.cosx_k(mol, coords, weights, dm, om)
        rel = np.max(np.abs(K[j] - Kref)) / np.abs(Kref).max()
        assert rel < 1e-11, (om, rel)
        de = abs(0.25 * np.einsum('ij,ji->', dm, K[j] - Kref))
        assert de < 1e-11, (om, de)


def test_fp64_k_f_shells_drug_like():
    """f shells (the rolled f-class kernels) on a seeded drug-like molecule
    (C, N, O, S, F, Cl, H) in the synthetic TZVP basis."""
    from pyscf_wb97mv_fast_gb300.basis import Molecule
    from pyscf_wb97mv_fast_gb300.systems import drug_like
    mol = Molecule.build(drug_like(0), 'synthetic-tzvp')
    coords, weights = grid_subset(mol, 1, 600, 4)
    dm = density(mol.nao, 30, 5)
    K, _ = _k64(mol, coords, weights, dm, (0.3, 0.0))
    for j, om in enumerate((0.3, 0.0)):
        Kref = oracle.cosx_k(mol, coords, weights, dm, om)
        rel = np.max(np.abs(K[j] - Kref)) / np.abs(Kref).max()
        assert rel < 1e-11, (om, rel)


def test_fp64_counters_reproducibility_and_mixed_agreement():
    """Model-flop counters equal the per-pair table times the points; two
    calls agree bitwise; the mixed-precision K agrees with the FP64 form
    within the mixed-precision gate."""
    torch = _torch()
    from pyscf_wb97mv_fast_gb300.cosx import CosxEngine
    mol = dimer('synthetic-svp')
    coords, weights = grid_subset(mol, 1, 2500, 7)
    dm = density(mol.nao, 10, 8)
    eng = CosxEngine(mol)
    K1, st = _k64(mol, coords, weights, dm, (0.0, 0.3), eng=eng)
    K2, _ = _k64(mol, coords, weights, dm, (0.0, 0.3), eng=eng)
    assert np.array_equal(K1, K2)
    pairs = eng.pair_table()
    per_point = float(pairs[:, 7].sum())
    assert st['model_flops'] == pytest.approx(2 * len(coords) * per_point, rel=1e-12)
    c = eng.relative(coords)
    w = torch.as_tensor(weights, device=eng.device)
    qd = torch.as_tensor(dm, device=eng.device)
    Km = eng.get_k_multi(c, w, qd, (0.0, 0.3), tile_tol=0.0)
    Km = ((Km + Km.transpose(1, 2)) * 0.5).cpu().numpy()
    for j in range(2):
        assert np.max(np.abs(Km[j] - K1[j])) < 1e-6 * np.abs(K1[j]).max()


def test_fp64_screening_error():
    """Screened (1e-11) vs unscreened FP64 K on 8 waters with a per-water
    localised density: the same bounds as the mixed-precision screen."""
    mol = waters(8, 7.0, 8)
    coords, weights = grid_subset(mol, 1, 6000, 5)
    dm = local_density(mol, seed=5)
    K0, s0 = _k64(mol, coords, weights, dm, (0.0,), tile_tol=0.0)
    K1, s1 = _k64(mol, coords, weights, dm, (0.0,), tile_tol=1e-11)
    assert s0['pairs_kept'] == s0['pairs_total']
    assert s1['pairs_kept'] < s1['pairs_total']
    assert np.max(np.abs(K1 - K0)) < 5e-8
    assert abs(0.25 * np.einsum('ij,ji->', dm, K1[0] - K0[0])) < 1e-8


def test_fp64_empty_grid_and_bad_arguments():
    torch = _torch()
    from pyscf_wb97mv_fast_gb300 import _native
    from pyscf_wb97mv_fast_gb300.cosx import CosxEngine
    mol = dimer('synthetic-svp')
    eng = CosxEngine(mol)
    qd = torch.as_tensor(density(mol.nao, 5, 0), device=eng.device)
    c = torch.zeros((0, 3), dtype=torch.float64, device=eng.device)
    w = torch.zeros((0,), dtype=torch.float64, device=eng.device)
    K = eng.get_k_fp64(c, w, qd, (0.0,))
    assert torch.count_nonzero(K).item() == 0
    with pytest.raises(_native.NativeError):
        eng.get_k_fp64(c, w, qd, (-1.0,))


def test_mixed_path_against_fp64_form_water27():
    """The bench molecule at full size (27 waters, synthetic def2-SVP, 648
    AOs, level-1 grid): the mixed-precision multi-omega build against the
    plain FP64 form on the same screen setting.  Gates: max|dK| < 1e-6
    max|K| and |1/4 tr(D dK)| below the reference's water27 floor of an
    FP32 full-K build (3e-6; README.md known issue 1)."""
    import torch
    from pyscf_wb97mv_fast_gb300.basis import Molecule
    from pyscf_wb97mv_fast_gb300.cosx import CosxEngine
    from pyscf_wb97mv_fast_gb300.grids import build_grids
    from pyscf_wb97mv_fast_gb300.systems import water_cluster
    mol = Molecule.build(water_cluster(27, box=10.0, seed=27), 'synthetic-svp')
    g = build_grids(mol, level=1)
    dm = local_density(mol, seed=27)
    eng = CosxEngine(mol)
    c = eng.relative(g.coords)
    w = torch.as_tensor(g.weights, device=eng.device)
    qd = torch.as_tensor(dm, device=eng.device)
    Km = eng.get_k_multi(c, w, qd, (0.0, 0.3), tile_tol=1e-11)
    Km = ((Km + Km.transpose(1, 2)) * 0.5).cpu().numpy()
    K64, _ = _k64(mol, g.coords, g.weights, dm, (0.0, 0.3), tile_tol=1e-11, eng=eng)
    for j in range(2):
        scale = np.abs(K64[j]).max()
        assert np.max(np.abs(Km[j] - K64[j])) < 1e-6 * scale
        assert abs(0.25 * np.einsum('ij,ji->', dm, Km[j] - K64[j])) < 3e-6


def test_builder_fp64_precision_for_the_tail():
    """GpuKBuilder(precision='fp64'), the K of an FP64 tail on the GPU
    (install_gpu(k_precision='fp64'), StagedSCF(fp64_final_k='gpu')): the
    reference's get_k contract, FP64 agreement with the oracle, and the
    second omega of a cycle served from the multi-omega build."""
    from pyscf_wb97mv_fast_gb300.gpu.sgx_k import (GpuKBuilder, SyntheticSGX,
                                                   get_k_only_gpu)
    from pyscf_wb97mv_fast_gb300.grids import build_grids
    mol = dimer('synthetic-svp')
    g = build_grids(mol, level=0)
    sgx = SyntheticSGX(mol, g)
    dm = density(mol.nao, 10, 9)
    b = GpuKBuilder(mol, tile_tol=0.0, precision='fp64', omegas=(0.0, 0.3))
    K0 = get_k_only_gpu(b, sgx, dm)
    assert np.array_equal(K0, K0.T)
    mol.omega = 0.3
    try:
        K3 = get_k_only_gpu(b, sgx, dm)
        assert b.last_stats['from_multi']
    finally:
        mol.omega = 0.0
    for K, om in ((K0, 0.0), (K3, 0.3)):
        ref = oracle.cosx_k(mol, g.coords, g.weights, dm, om)
        assert np.max(np.abs(K - ref)) < 1e-11 * np.abs(ref).max()
    with pytest.raises(ValueError):
        GpuKBuilder(mol, precision='fp16')
