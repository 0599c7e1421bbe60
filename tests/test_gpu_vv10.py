"""VV10 on the GPU vs the FP64 oracle and the reference (reference tests:
tests/gpu/test_xc_vv10.py:116-152, :275-343)."""
import os
import time

import numpy as np
import pytest

import oracle
from helpers import dimer

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), 'golden')

pytestmark = pytest.mark.gpu


def _kernel_sum(coords, q, w0, kappa, tile_tol=0.0):
    import torch
    from pyscf_wb97mv_fast_gb300.gpu.vv10 import Vv10Kernel
    k = Vv10Kernel(tile_tol)
    out = k.kernel_sum(torch.as_tensor(coords, dtype=torch.float32, device='cuda'),
                       torch.as_tensor(q, device='cuda'),
                       torch.as_tensor(w0, device='cuda'),
                       torch.as_tensor(kappa, device='cuda'))
    return [o.cpu().numpy() for o in out], k.last_pairs_kept


def _points(n, seed):
    rng = np.random.default_rng(seed)
    return (rng.uniform(-6, 6, (n, 3)), rng.uniform(1e-4, 1e-2, n),
            rng.uniform(0.3, 3.0, n), rng.uniform(0.4, 2.0, n))


def test_kernel_sum_matches_fp64_bruteforce():
    """Relative error <= 1e-6 on F, U, W against the FP64 sum of the same
    (FP32-representable) inputs; 1100 points: several 256-point tiles and a
    ragged tail."""
    c, q, w0, k = (a.astype(np.float32).astype(np.float64) for a in _points(1100, 0))
    (F, U, W), kept = _kernel_sum(c, q, w0, k)
    ref = oracle.vv10_sum(c, q, w0, k)
    for got, r, name in zip((F, U, W), ref, 'FUW'):
        assert got.dtype == np.float64
        rel = np.abs(got - r) / np.abs(r)
        assert rel.max() < 1e-6, (name, rel.max())
    assert kept == (1100 * 1100, 1100 * 1100)


def test_kernel_sum_matches_reference_golden():
    d = np.load(os.path.join(GOLDEN, 'vv10.npz'))
    (F, U, W), _ = _kernel_sum(d['xyz'], d['q'], d['w0'], d['kappa'])
    for got, r in ((F, d['F']), (U, d['U']), (W, d['W'])):
        assert np.max(np.abs(got - r) / np.abs(r)) < 1e-5


def test_kernel_sum_bitwise_reproducible():
    c, q, w0, k = _points(3000, 1)
    a, _ = _kernel_sum(c, q, w0, k)
    b, _ = _kernel_sum(c, q, w0, k)
    for x, y in zip(a, b):
        assert np.array_equal(x, y)


def test_tile_pruning_drops_only_negligible_pairs():
    """Two clusters 1000 bohr apart: pruned and exact sums agree to 1e-6,
    and pairs are dropped (reference :320-343)."""
    rng = np.random.default_rng(7)
    n = 1024
    a = rng.uniform(-2, 2, (n, 3))
    b = rng.uniform(-2, 2, (n, 3)) + np.array([1000.0, 0.0, 0.0])
    c = np.concatenate([a, b])
    q = rng.uniform(1e-4, 1e-3, 2 * n)
    w0 = rng.uniform(0.5, 2.0, 2 * n)
    k = rng.uniform(0.5, 2.0, 2 * n)
    ref, kept0 = _kernel_sum(c, q, w0, k, 0.0)
    got, kept1 = _kernel_sum(c, q, w0, k, 1e-12)
    assert kept1[0] < kept1[1] and kept0[0] == kept0[1]
    for g, r in zip(got, ref):
        assert np.max(np.abs(g - r) / np.abs(r)) < 1e-6


def test_kernel_sum_throughput_floor():
    """> 1e10 pairs/s at n = 65536 (reference floor, test_xc_vv10.py:296)."""
    import torch
    from pyscf_wb97mv_fast_gb300.gpu.vv10 import Vv10Kernel
    rng = np.random.default_rng(0)
    n = 65536
    args = [torch.as_tensor(rng.uniform(-10, 10, (n, 3)), dtype=torch.float32,
                            device='cuda'),
            torch.as_tensor(rng.uniform(1e-4, 1e-2, n), device='cuda'),
            torch.as_tensor(rng.uniform(0.5, 3, n), device='cuda'),
            torch.as_tensor(rng.uniform(0.5, 2, n), device='cuda')]
    kern = Vv10Kernel(0.0)
    kern.kernel_sum(*args)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    kern.kernel_sum(*args)
    torch.cuda.synchronize()
    rate = n * n / (time.perf_counter() - t0)
    assert rate > 1e10, '%.3e pairs/s' % rate


def test_ao_deriv1_matches_reference():
    from pyscf_wb97mv_fast_gb300.cosx import CosxEngine
    for tag, basis in (('svp', 'synthetic-svp'), ('tzvp', 'synthetic-tzvp')):
        d = np.load(os.path.join(GOLDEN, 'int3c1e_%s.npz' % tag))
        eng = CosxEngine(dimer(basis))
        n = len(d['ao_coords'])
        X = eng.ao_eval_deriv1(eng.relative(d['ao_coords'])).cpu().numpy()[:, :, :n]
        ref = d['ao1'].transpose(0, 2, 1)
        assert np.max(np.abs(X - ref)) < 1e-13 * np.abs(ref).max()


def test_nr_nlc_vxc_matches_reference_flow():
    """gpu_nr_nlc_vxc vs the reference's flow (golden) and the FP64 oracle:
    |d nelec| < 1e-10, |d E_nlc| < 1e-8, max |d vmat| < 1e-7."""
    import types
    from pyscf_wb97mv_fast_gb300.gpu.vv10 import Vv10Context, gpu_nr_nlc_vxc
    d = np.load(os.path.join(GOLDEN, 'vv10_flow.npz'))
    mol = dimer()
    pars = [((float(d['nlc_b']), float(d['nlc_c'])), 1.0)]
    ni = types.SimpleNamespace(nlc_coeff=lambda xc: pars)
    grids = types.SimpleNamespace(coords=d['coords'], weights=d['weights'])
    ctx = Vv10Context(mol)
    n, e, v = gpu_nr_nlc_vxc(ctx, ni, mol, grids, 'wb97m-v', d['dm'])
    n0, e0, v0 = oracle.nlc_vxc(mol, d['coords'], d['weights'], d['dm'], pars)
    for (nn, ee, vv) in ((d['nelec'], d['exc'], d['vmat']), (n0, e0, v0)):
        assert abs(n - nn) < 1e-10
        assert abs(e - ee) < 1e-8
        assert np.max(np.abs(v - vv)) < 1e-7


@pytest.mark.parametrize('tile_tol', [0.0, 1e-12])
def test_batched_kernel_sum_equals_per_molecule(tile_tol):
    """Several molecules' point sets in one launch (ragged sizes, one below
    a tile, one of exactly two tiles): each molecule's F, U, W bitwise equal
    to its own single call, and the kept-pair counts add up."""
    import torch
    from pyscf_wb97mv_fast_gb300.gpu.vv10 import Vv10Kernel
    sets = [_points(n, 10 + i) for i, n in enumerate((700, 100, 512, 1301))]
    dev = 'cuda'
    cs = [torch.as_tensor(c, dtype=torch.float32, device=dev) for c, _, _, _ in sets]
    qs = [torch.as_tensor(q, device=dev) for _, q, _, _ in sets]
    ws = [torch.as_tensor(w, device=dev) for _, _, w, _ in sets]
    ks = [torch.as_tensor(k, device=dev) for _, _, _, k in sets]
    kb = Vv10Kernel(tile_tol)
    Fb, Ub, Wb = kb.kernel_sum_batch(cs, qs, ws, ks)
    kept = 0
    for i in range(len(sets)):
        k1 = Vv10Kernel(tile_tol)
        F, U, W = k1.kernel_sum(cs[i], qs[i], ws[i], ks[i])
        assert torch.equal(F, Fb[i]) and torch.equal(U, Ub[i]) and torch.equal(W, Wb[i])
        kept += k1.last_pairs_kept[0]
    assert kb.last_pairs_kept[0] == kept
    assert kb.last_pairs_kept[1] == sum(len(s[1]) ** 2 for s in sets)
