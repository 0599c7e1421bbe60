"""K parity on the reference's six validation molecules (caffeine,
sulfamethoxazole, bromazepam, ibuprofen, fluoxetine, chlorpromazine;
benchmarks/systems/drugs/*.xyz, README.md:118-128) in the synthetic
def2-TZVP structure (f shells; H, C, N, O, F, S, Cl, Br), against the FP64
oracle with the reference's gates (tests/gpu/test_sgx_k.py:24-69)."""
import numpy as np
import pytest

import oracle
from helpers import DRUGS, density, drug

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize('name', DRUGS)
def test_mixed_k_matches_oracle_on_drug(name):
    import torch
    from pyscf_wb97mv_fast_gb300.cosx import CosxEngine
    from pyscf_wb97mv_fast_gb300.grids import build_grids
    mol = drug(name)
    g = build_grids(mol, level=0)
    idx = np.sort(np.random.default_rng(3).choice(g.size, 500, replace=False))
    coords, w = g.coords[idx], g.weights[idx]
    dm = density(mol.nao, mol.nelectron // 2, seed=7)
    eng = CosxEngine(mol, device=0)
    K = eng.get_k_multi(eng.relative(coords), torch.as_tensor(w, device='cuda'),
                        torch.as_tensor(dm, device='cuda'), (0.0, 0.3),
                        tile_tol=1e-11)
    K = (0.5 * (K + K.transpose(1, 2))).cpu().numpy()
    for j, (omega, gate) in enumerate(((0.0, 3e-7), (0.3, 1e-7))):
        ref = oracle.cosx_k(mol, coords, w, dm, omega)
        dk = K[j] - ref
        assert np.abs(dk).max() < 1e-6 * np.abs(ref).max(), (name, omega)
        assert abs(0.25 * float(np.sum(dm * dk))) < gate, (name, omega)
