"""The F product on this library's tcgen05 tensor-core kernel (ozaki_tc.cu:
TMA loads, MMAs into TMEM, the level combination in the epilogue) against
the cuBLAS level-GEMM form of the same Ozaki split: the FP32 level sums are
exact integers in any summation order, so the two engines give bitwise the
same F; and F against FP64 X QD rounded to FP32."""
import numpy as np
import pytest

from helpers import density, dimer, waters

pytestmark = pytest.mark.gpu


def _case(mol, npts, seed):
    import torch
    from pyscf_wb97mv_fast_gb300.cosx import CosxEngine, round32
    from pyscf_wb97mv_fast_gb300.grids import build_grids
    g = build_grids(mol, level=0)
    idx = np.sort(np.random.default_rng(seed).choice(g.size, min(npts, g.size),
                                                     replace=False))
    eng = CosxEngine(mol, device=0)
    c = eng.relative(g.coords[idx])
    X = eng.ao_eval(c)
    dm = torch.as_tensor(density(mol.nao, max(2, mol.nao // 6), seed), device='cuda')
    return eng, X, dm


@pytest.mark.parametrize('name', ['dimer_svp', 'dimer_tzvp', 'dimer_gen', 'waters6'])
def test_tc_engine_is_bitwise_the_library_engine(name):
    import torch
    from pyscf_wb97mv_fast_gb300 import cosx
    mol = {'dimer_svp': lambda: dimer('synthetic-svp'),
           'dimer_tzvp': lambda: dimer('synthetic-tzvp'),
           'dimer_gen': lambda: dimer('synthetic-svp', True),
           'waters6': lambda: waters(6, box=8.0, seed=4)}[name]()
    eng, X, dm = _case(mol, 3000, 7)
    prev = cosx.set_f_engine('tc')
    try:
        F_tc = eng.ozaki_f(X, dm)
        cosx.set_f_engine('library')
        F_lib = eng.ozaki_f(X, dm)
    finally:
        cosx.set_f_engine(prev)
    torch.cuda.synchronize()
    assert not torch.isnan(F_tc).any()
    assert torch.equal(F_tc, F_lib), name
    # and F is fl32 of the FP64 product to FP32 rounding
    ref = dm.T @ X
    scale = ref.abs().amax(dim=0, keepdim=True).clamp_min(1e-300)
    assert float(((F_tc.to(torch.float64) - ref).abs() / scale).max()) < 1e-6


def test_tc_engine_in_the_k_build_matches_library_engine():
    """A whole multi-omega K build with each engine: the same F makes the
    same G and K, bitwise."""
    import torch
    from pyscf_wb97mv_fast_gb300 import cosx
    mol = waters(4, box=6.0, seed=11)
    eng, X, dm = _case(mol, 5000, 3)
    from pyscf_wb97mv_fast_gb300.grids import build_grids
    g = build_grids(mol, level=0)
    c = eng.relative(g.coords[:5000])
    w = torch.as_tensor(g.weights[:5000], device='cuda')
    prev = cosx.get_f_engine()
    try:
        out = {}
        for e in ('tc', 'library'):
            cosx.set_f_engine(e)
            out[e] = eng.get_k_multi(c, w, dm, (0.0, 0.3), tile_tol=1e-11)
    finally:
        cosx.set_f_engine(prev)
    assert torch.equal(out['tc'], out['library'])
    assert cosx.get_f_engine() == prev


@pytest.mark.parametrize('engine', ['tc', 'library'])
def test_fp64_output_split_is_42_bit_accurate(engine):
    """wb_cosx_ozaki_f64 / _k64 (the SCF FP64 tail's quadrature GEMMs):
    within 2^-40 of the per-point / per-column maxima of an FP64 product,
    and the two F engines agree bitwise."""
    import torch
    from pyscf_wb97mv_fast_gb300 import cosx
    mol = dimer('synthetic-tzvp')
    eng, X, dm = _case(mol, 4000, 5)
    prev = cosx.set_f_engine(engine)
    try:
        F64 = eng.ozaki_f(X, dm, fp64=True)
        cosx.set_f_engine('library' if engine == 'tc' else 'tc')
        F64b = eng.ozaki_f(X, dm, fp64=True)
    finally:
        cosx.set_f_engine(prev)
    assert F64.dtype == torch.float64
    assert torch.equal(F64, F64b)
    ref = dm.T @ X
    bound = (X.abs().amax(dim=0, keepdim=True) *
             dm.abs().amax(dim=0)[:, None]) * mol.nao * 2.0 ** -40
    assert bool(((F64 - ref).abs() <= bound + 1e-300).all())
    # K side with an FP64 G: X^T (w o G)
    n = X.shape[1]
    w = torch.rand(n, dtype=torch.float64, device='cuda') + 0.5
    G = torch.randn_like(X)
    K = eng.ozaki_k(X, G, w)
    Kref = X @ (w[None, :] * G).T
    scale = float(X.abs().max()) * float((w[None, :] * G).abs().max()) * n
    assert float((K - Kref).abs().max()) < scale * 2.0 ** -40
