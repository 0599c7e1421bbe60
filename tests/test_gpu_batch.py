"""Batched K builds (wb_cosx_batch_*): several molecules per call, one
launch per class kernel over all of them.  Each molecule's K against its
own single-molecule build (wb_cosx_get_k_multi) and the FP64 oracle; CUDA
graph capture of a batched run.  All calls go through the C ABI."""
import numpy as np
import pytest

import oracle
from helpers import density, dimer, grid_subset, waters

pytestmark = pytest.mark.gpu


def _setup(mols, npts, seed):
    import torch
    from pyscf_wb97mv_fast_gb300.cosx import CosxEngine
    engines, grids, dms, raw = [], [], [], []
    for i, mol in enumerate(mols):
        eng = CosxEngine(mol)
        coords, weights = grid_subset(mol, 0, npts, seed + i)
        grids.append((eng.relative(coords), torch.as_tensor(weights, device=eng.device)))
        dm = density(mol.nao, 6, seed + 10 + i)
        dms.append(torch.as_tensor(dm, device=eng.device))
        engines.append(eng)
        raw.append((mol, coords, weights, dm))
    return engines, grids, dms, raw


def _single(mol, coords, weights, dm, omegas):
    import torch
    from pyscf_wb97mv_fast_gb300.cosx import CosxEngine
    eng = CosxEngine(mol)
    K = eng.get_k_multi(eng.relative(coords), torch.as_tensor(weights, device=eng.device),
                        torch.as_tensor(dm, device=eng.device), omegas, tile_tol=1e-11)
    return K.cpu().numpy(), eng.last_stats


def test_batch_of_waters_equals_single_builds_bitwise():
    from pyscf_wb97mv_fast_gb300.cosx import CosxBatch
    mols = [waters(3, 5.0, 1), waters(5, 6.0, 2), dimer('synthetic-svp'),
            waters(4, 5.5, 3)]
    engines, grids, dms, raw = _setup(mols, 3000, 40)
    b = CosxBatch(engines, grids, (0.0, 0.3), tile_tol=1e-11)
    Ks = b.run(dms, stats=True)
    flops = 0.0
    for K, (mol, c, w, dm) in zip(Ks, raw):
        Kref, st = _single(mol, c, w, dm, (0.0, 0.3))
        assert np.array_equal(K.cpu().numpy(), Kref)
        flops += st['model_flops']
    assert b.last_stats['model_flops'] == flops
    # a second run with other densities reuses the plan
    dms2 = [d.flip(0).flip(1).contiguous() for d in dms]
    Ks2 = b.run(dms2)
    for K, (mol, c, w, _), d in zip(Ks2, raw, dms2):
        Kref, _ = _single(mol, c, w, d.cpu().numpy(), (0.0, 0.3))
        assert np.array_equal(K.cpu().numpy(), Kref)
    b.close()


def test_mixed_batch_matches_oracle():
    """Molecules with different shell structures in one batch (an alkane
    with f shells next to waters, general contractions): each K within the
    reference's K gate of the FP64 oracle."""
    from pyscf_wb97mv_fast_gb300.basis import Molecule
    from pyscf_wb97mv_fast_gb300.cosx import CosxBatch
    from pyscf_wb97mv_fast_gb300.systems import alkane
    mols = [Molecule.build(alkane(4), 'synthetic-tzvp'), waters(3, 5.0, 4),
            dimer('synthetic-svp', True)]
    engines, grids, dms, raw = _setup(mols, 1500, 60)
    b = CosxBatch(engines, grids, (0.3, 0.0), tile_tol=0.0)
    Ks = b.run(dms)
    for K, (mol, c, w, dm) in zip(Ks, raw):
        K = K.cpu().numpy()
        for j, om in enumerate((0.3, 0.0)):
            Kj = (K[j] + K[j].T) * 0.5
            ref = oracle.cosx_k(mol, c, w, dm, om)
            assert np.max(np.abs(Kj - ref)) < 1e-6 * np.abs(ref).max()
            gate = 3e-7 if om == 0.0 else 1e-7
            assert abs(0.25 * np.einsum('ij,ji->', dm, Kj - ref)) < gate
    b.close()


def test_single_omega_batch_and_graph_capture():
    import torch
    from pyscf_wb97mv_fast_gb300.cosx import CosxBatch
    mols = [waters(3, 5.0, 7), dimer('synthetic-svp')]
    engines, grids, dms, raw = _setup(mols, 2000, 80)
    b1 = CosxBatch(engines, grids, (0.3,), tile_tol=1e-11)
    for K, (mol, c, w, dm) in zip(b1.run(dms), raw):
        Kref, _ = _single(mol, c, w, dm, (0.3,))
        assert np.max(np.abs(K.cpu().numpy() - Kref)) < 1e-12 * np.abs(Kref).max()
    b1.close()
    # a two-omega batch captured in a CUDA graph: replays equal direct runs
    b = CosxBatch(engines, grids, (0.0, 0.3), tile_tol=1e-11)
    qd = [torch.zeros_like(d) for d in dms]
    out = b.run(dms)                                   # warm-up
    torch.cuda.synchronize()
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g):
        b.run(qd, out=out)
    for src in (dms, [d * 0.5 for d in dms]):
        for q, d in zip(qd, src):
            q.copy_(d)
        g.replay()
        direct = b.run(src)
        for a, c in zip(out, direct):
            assert torch.equal(a, c)
    b.close()


def test_batch_argument_errors():
    from pyscf_wb97mv_fast_gb300 import _native
    from pyscf_wb97mv_fast_gb300.cosx import CosxBatch
    mols = [dimer('synthetic-svp')]
    engines, grids, dms, _ = _setup(mols, 500, 90)
    with pytest.raises(_native.NativeError):
        CosxBatch(engines + engines, grids + grids, (0.0,))      # one handle twice
    with pytest.raises(ValueError):
        CosxBatch(engines, grids, (0.0, 0.1, 0.3))
    b = CosxBatch(engines, grids, (0.0,))
    with pytest.raises(ValueError):
        b.run(dms + dms)
    b.close()
