"""The fused device screen keeps a superset of the reference's FP64 screen
(reference test: tests/gpu/test_sgx_k.py:166-206).

The G kernels screen each (point block, shell pair) task with an FP32 bound
inflated to stay above the exact one.  Here the device's kept set
(wb_cosx_screen_mask: the same screen function on the same block statistics
and pair data as the class kernels) is compared with the oracle's FP64
restatement of the reference's locked bound (pair_bound times the F
estimate, gpu/shellpairs.py:545-555, gpu/sgx_k.py:926-958) on the same FP32
F: every task the FP64 bound keeps must be kept on the device, and the
extra ones -- estimates within ~0.1 % of the tolerance -- must be rare.
"""
import numpy as np
import pytest

import oracle
from helpers import density, dimer, waters

pytestmark = pytest.mark.gpu


def _device_and_oracle(mol, tol, level, nocc=10, seed=0):
    import torch
    from pyscf_wb97mv_fast_gb300.cosx import CosxEngine, round32
    from pyscf_wb97mv_fast_gb300.grids import build_grids
    g = build_grids(mol, level=0)
    coords, w = g.coords, g.weights
    D = density(mol.nao, nocc, seed)
    F32 = (oracle.ao_eval(mol, coords) @ D).astype(np.float32)   # (ng, nao)
    eng = CosxEngine(mol, device=0)
    ld = round32(len(coords))
    f = torch.zeros((mol.nao, ld), dtype=torch.float32, device='cuda')
    f[:, :len(coords)] = torch.as_tensor(F32.T.copy(), device='cuda')
    keep_dev = eng.screen_mask(eng.relative(coords),
                               torch.as_tensor(w, device='cuda'), f, tol,
                               level).cpu().numpy().astype(bool)
    table = eng.pair_table()
    # virtual shells are the physical ones for bases without general
    # contractions; orient each pair as the reference does (ish >= jsh)
    dev_pairs = [(int(max(a, b)), int(min(a, b))) for a, b in table[:, 5:7]]
    keep_ref, ref_pairs = oracle.screen_keep_fp64(mol, coords, w, F32, tol,
                                                  block_pts=32 << level)
    return keep_dev, dev_pairs, keep_ref, ref_pairs


@pytest.mark.parametrize('tol', [1e-11, 1e-7, 1e-5])
@pytest.mark.parametrize('basis', ['synthetic-svp', 'synthetic-tzvp'])
def test_device_screen_keeps_superset_of_fp64_bound(basis, tol):
    mol = dimer(basis)
    keep_dev, dev_pairs, keep_ref, ref_pairs = _device_and_oracle(mol, tol, 0)
    assert sorted(dev_pairs) == sorted(ref_pairs)     # the same 1e-14 pair cut
    col = {p: k for k, p in enumerate(dev_pairs)}
    dev = keep_dev[:, [col[p] for p in ref_pairs]]
    assert dev.shape == keep_ref.shape
    missed = keep_ref & ~dev
    assert not missed.any(), (basis, tol, int(missed.sum()))
    extra = int((dev & ~keep_ref).sum())
    assert extra <= max(2, 1e-3 * dev.size), (basis, tol, extra, dev.size)
    # the screen does work at these tolerances
    if tol >= 1e-7:
        assert keep_ref.mean() < 0.9


@pytest.mark.parametrize('level', [1, 2])
def test_device_screen_superset_on_larger_blocks(level):
    """The 64- and 128-point blocks of the light classes' kernels, on a
    cluster where distant pairs are screened."""
    mol = waters(4, box=6.0, seed=3)
    keep_dev, dev_pairs, keep_ref, ref_pairs = _device_and_oracle(mol, 1e-11, level,
                                                                  nocc=20)
    col = {p: k for k, p in enumerate(dev_pairs)}
    dev = keep_dev[:, [col[p] for p in ref_pairs]]
    assert not (keep_ref & ~dev).any()
    assert int((dev & ~keep_ref).sum()) <= max(2, 1e-3 * dev.size)
    assert keep_ref.mean() < 0.95
