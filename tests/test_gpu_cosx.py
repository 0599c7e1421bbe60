"""COSX kernels on the GPU vs the FP64 oracle and the reference's golden
vectors (reference tests: tests/gpu/test_boys.py, test_int3c1e.py,
test_sgx_k.py, test_ao_eval.py).  All calls go through the C ABI."""
import os

import numpy as np
import pytest
from scipy.special import gamma, gammainc

import oracle
from helpers import density, dimer, grid_subset, local_density, waters

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), 'golden')

pytestmark = pytest.mark.gpu


def _torch():
    import torch
    return torch


def ref_boys(n, T):
    T = np.asarray(T, dtype=np.float64)
    out = np.empty_like(T)
    small = T < 1e-12
    out[small] = 1.0 / (2 * n + 1)
    Ts = T[~small]
    out[~small] = gamma(n + 0.5) * gammainc(n + 0.5, Ts) / (2.0 * Ts ** (n + 0.5))
    return out


# -- Boys -----------------------------------------------------------------------

def test_boys_fp32_relative_error():
    torch = _torch()
    from pyscf_wb97mv_fast_gb300.cosx import boys_eval
    T = np.concatenate([[0.0, 1e-30, 1e-8], np.linspace(0, 50, 20001),
                        np.geomspace(50, 1e6, 2000)]).astype(np.float32)
    F = boys_eval(torch.as_tensor(T, device='cuda'), 6).cpu().numpy()
    for n in range(7):
        ref = ref_boys(n, T.astype(np.float64))
        rel = np.abs(F[n] - ref) / ref
        assert np.all(np.isfinite(F[n]))
        assert rel.max() < 2e-7, (n, rel.max(), T[rel.argmax()])


def test_boys_fp32_unbiased():
    """Mean signed relative error over T in [0, 50] << FP32 eps (a biased
    F_n biases every integral the same way)."""
    torch = _torch()
    from pyscf_wb97mv_fast_gb300.cosx import boys_eval
    T = np.random.default_rng(0).uniform(0, 50, 1_000_000).astype(np.float32)
    F = boys_eval(torch.as_tensor(T, device='cuda'), 6).cpu().numpy()
    for n in range(7):
        ref = ref_boys(n, T.astype(np.float64))
        assert abs(np.mean((F[n] - ref) / ref)) < 1e-8, n


def test_boys_nmax_slices_and_range():
    torch = _torch()
    from pyscf_wb97mv_fast_gb300.cosx import boys_eval
    T = torch.as_tensor(np.linspace(0, 40, 101).astype(np.float32), device='cuda')
    full = boys_eval(T, 6).cpu().numpy()
    for nmax in (0, 2, 4, 6):
        part = boys_eval(T, nmax).cpu().numpy()
        assert part.shape == (nmax + 1, 101)
        assert np.array_equal(part, full[:nmax + 1])
    with pytest.raises(ValueError):
        boys_eval(T, 7)


# -- dense integrals and AO values vs the reference's own FP64 code -----------

@pytest.mark.parametrize('tag,basis,gen', [('svp', 'synthetic-svp', False),
                                           ('tzvp', 'synthetic-tzvp', False),
                                           ('gen', 'synthetic-svp', True)])
@pytest.mark.parametrize('omega', [0.0, 0.3])
def test_dense_int3c1e_matches_reference(tag, basis, gen, omega):
    from pyscf_wb97mv_fast_gb300.cosx import CosxEngine
    d = np.load(os.path.join(GOLDEN, 'int3c1e_%s.npz' % tag))
    mol = dimer(basis, gen)
    eng = CosxEngine(mol)
    got = eng.int3c1e_dense(eng.relative(d['coords']), omega).cpu().numpy()
    ref = d['A_w%g' % omega]
    assert np.all(np.isfinite(got))
    assert np.max(np.abs(got - ref)) < 1e-6 * np.abs(ref).max()
    big = np.abs(ref) > 1e-3 * np.abs(ref).max()
    assert abs(np.mean((got[big] - ref[big]) / ref[big])) < 1e-7
    assert np.array_equal(got, got.transpose(0, 2, 1))
    again = eng.int3c1e_dense(eng.relative(d['coords']), omega).cpu().numpy()
    assert np.array_equal(got, again)


@pytest.mark.parametrize('tag,basis,gen', [('svp', 'synthetic-svp', False),
                                           ('tzvp', 'synthetic-tzvp', False),
                                           ('gen', 'synthetic-svp', True)])
def test_ao_eval_matches_reference(tag, basis, gen):
    from pyscf_wb97mv_fast_gb300.cosx import CosxEngine
    d = np.load(os.path.join(GOLDEN, 'int3c1e_%s.npz' % tag))
    eng = CosxEngine(dimer(basis, gen))
    n = len(d['ao_coords'])
    X = eng.ao_eval(eng.relative(d['ao_coords'])).cpu().numpy()[:, :n].T
    ref = d['ao']
    assert np.max(np.abs(X - ref)) < 1e-13 * np.abs(ref).max()


# -- fused G kernels vs the FP64 oracle ----------------------------------------

def _g_case(mol, npts, seed, omega, tile_tol=0.0):
    torch = _torch()
    from pyscf_wb97mv_fast_gb300.cosx import CosxEngine, round32
    eng = CosxEngine(mol)
    coords, weights = grid_subset(mol, 1, npts, seed)
    n = len(coords)
    X = oracle.ao_eval(mol, coords)
    dm = density(mol.nao, 10, seed)
    F32 = (X @ dm).astype(np.float32)
    ld = round32(n)
    Fd = torch.zeros((mol.nao, ld), dtype=torch.float32, device=eng.device)
    Fd[:, :n] = torch.as_tensor(F32.T, device=eng.device)
    w = torch.as_tensor(weights, device=eng.device)
    G = eng.g(eng.relative(coords), w, Fd, omega, tile_tol).cpu().numpy()[:, :n].T
    Gref = oracle.cosx_g(mol, coords, F32.astype(np.float64), omega)
    return eng, G, Gref, n


@pytest.mark.parametrize('basis,gen', [('synthetic-svp', False),
                                       ('synthetic-tzvp', False),
                                       ('synthetic-svp', True)])
@pytest.mark.parametrize('omega', [0.0, 0.3])
def test_g_kernels_match_oracle(basis, gen, omega):
    mol = dimer(basis, gen)
    eng, G, Gref, n = _g_case(mol, 700, 3, omega)
    scale = np.abs(Gref).max()
    assert np.all(np.isfinite(G))
    assert np.max(np.abs(G - Gref)) < 2e-6 * scale, np.max(np.abs(G - Gref)) / scale
    st = eng.last_stats
    assert st['pairs_kept'] == st['pairs_total']          # tile_tol = 0
    # counters: model flops / integrals are exact sums over the pair table
    rows = eng.pair_table()
    nsub_full, rem = divmod(n, 32)
    pts = 32 * nsub_full + rem
    assert st['model_flops'] == float(rows[:, 7].sum() * pts)


def test_g_kernels_bitwise_reproducible():
    mol = dimer('synthetic-tzvp')
    _, G1, _, _ = _g_case(mol, 900, 4, 0.3)
    _, G2, _, _ = _g_case(mol, 900, 4, 0.3)
    assert np.array_equal(G1, G2)


def test_block_order_does_not_change_g():
    """The first G launch on a grid takes the point blocks in ascending
    order, later ones costliest first (learnt from the previous launch):
    bitwise the same G and the same kept tasks, on one handle."""
    torch = _torch()
    from pyscf_wb97mv_fast_gb300.cosx import CosxEngine, round32
    mol = waters(4, 6.0, 12)
    eng = CosxEngine(mol)
    coords, weights = grid_subset(mol, 1, 20000, 9)
    n = len(coords)
    dm = density(mol.nao, 12, 9)
    F = (oracle.ao_eval(mol, coords) @ dm).astype(np.float32)
    Fd = torch.zeros((mol.nao, round32(n)), dtype=torch.float32, device=eng.device)
    Fd[:, :n] = torch.as_tensor(F.T, device=eng.device)
    c = eng.relative(coords)
    w = torch.as_tensor(weights, device=eng.device)
    runs = []
    for _ in range(3):
        G = eng.g_multi(c, w, Fd, (0.0, 0.3), 1e-11)
        runs.append((G.clone(), eng.last_stats['pairs_kept']))
    for G, kept in runs[1:]:
        assert torch.equal(G, runs[0][0])
        assert kept == runs[0][1]


# -- full K build vs the oracle and the reference --------------------------------

def _k_gpu(mol, coords, weights, dm, omega, tile_tol=0.0, tile_pts=0,
           gemm='ozaki'):
    torch = _torch()
    from pyscf_wb97mv_fast_gb300.cosx import CosxEngine
    eng = CosxEngine(mol)
    c = eng.relative(coords)
    w = torch.as_tensor(weights, device=eng.device)
    qd = torch.as_tensor(dm, device=eng.device)
    K = eng.get_k(c, w, qd, omega, tile_tol=tile_tol, tile_pts=tile_pts,
                  gemm=gemm)
    K = ((K + K.T) * 0.5).cpu().numpy()
    return K, eng.last_stats


@pytest.mark.parametrize('basis,gen', [('synthetic-svp', False),
                                       ('synthetic-tzvp', False),
                                       ('synthetic-svp', True)])
@pytest.mark.parametrize('omega', [0.0, 0.3])
def test_k_matches_oracle(basis, gen, omega):
    """Reference gate (tests/gpu/test_sgx_k.py:24-46): max|dK| < 1e-6
    max|K|, |1/4 tr(D dK)| < 3e-7 (full) / 1e-7 (long range), K exactly
    symmetric and bitwise reproducible."""
    mol = dimer(basis, gen)
    coords, weights = grid_subset(mol, 1, 4000, 1)
    dm = density(mol.nao, 10, 2)
    K1, st = _k_gpu(mol, coords, weights, dm, omega)
    K2, _ = _k_gpu(mol, coords, weights, dm, omega)
    Kref = oracle.cosx_k(mol, coords, weights, dm, omega)
    assert np.array_equal(K1, K2)
    assert np.array_equal(K1, K1.T)
    rel = np.max(np.abs(K1 - Kref)) / np.abs(Kref).max()
    assert rel < 1e-6, rel
    gate = 3e-7 if omega == 0.0 else 1e-7
    de = abs(0.25 * np.einsum('ij,ji->', dm, K1 - Kref))
    assert de < gate, de
    assert st['pairs_kept'] == st['pairs_total']


def _drug(seed, basis):
    from pyscf_wb97mv_fast_gb300.basis import Molecule
    from pyscf_wb97mv_fast_gb300.systems import drug_like
    return Molecule.build(drug_like(seed), basis)


@pytest.mark.parametrize('basis,npts', [('synthetic-svp', 3000),
                                        ('synthetic-tzvp', 1500)])
@pytest.mark.parametrize('omega', [0.0, 0.3])
def test_k_matches_oracle_drug_like(basis, npts, omega):
    """The K gates on a seeded drug-like molecule (C, N, O, S, F, Cl, H;
    f shells on every heavy atom in TZVP): the reference validates on drug
    molecules (README.md:118-128); here with synthetic molecules and basis
    data."""
    mol = _drug(0, basis)
    coords, weights = grid_subset(mol, 1, npts, 4)
    dm = density(mol.nao, 30, 5)
    K, st = _k_gpu(mol, coords, weights, dm, omega)
    Kref = oracle.cosx_k(mol, coords, weights, dm, omega)
    assert np.array_equal(K, K.T)
    rel = np.max(np.abs(K - Kref)) / np.abs(Kref).max()
    assert rel < 1e-6, rel
    gate = 3e-7 if omega == 0.0 else 1e-7
    de = abs(0.25 * np.einsum('ij,ji->', dm, K - Kref))
    assert de < gate, de


@pytest.mark.parametrize('omega', [0.0, 0.3])
def test_g_kernels_match_oracle_drug_like(omega):
    mol = _drug(1, 'synthetic-tzvp')
    _, G, Gref, _ = _g_case(mol, 600, 6, omega)
    assert np.max(np.abs(G - Gref)) < 2e-6 * np.abs(Gref).max()


@pytest.mark.parametrize('omega', [0.0, 0.3])
def test_k_matches_reference_golden(omega):
    """The reference's own FP64 K on the same 160 points (dense A from
    int3c1e_reference contracted as gpu/sgx_k.py:719-742)."""
    d = np.load(os.path.join(GOLDEN, 'k_svp.npz'))
    mol = dimer('synthetic-svp')
    K, _ = _k_gpu(mol, d['coords'], d['weights'], d['dm'], omega)
    ref = d['K_w%g' % omega]
    assert np.max(np.abs(K - ref)) < 1e-6 * np.abs(ref).max()


def test_k_tiles_do_not_change_result_beyond_rounding():
    mol = dimer('synthetic-svp')
    coords, weights = grid_subset(mol, 1, 5000, 3)
    dm = density(mol.nao, 10, 3)
    K1, _ = _k_gpu(mol, coords, weights, dm, 0.0)
    K2, st = _k_gpu(mol, coords, weights, dm, 0.0, tile_pts=1024)
    # the tile boundaries move the Ozaki chunk boundaries (per-chunk
    # scaling, 42 bits): agreement far below FP32 noise
    assert np.max(np.abs(K1 - K2)) < 1e-10 * np.abs(K1).max()
    assert st['kernel_launches'] > 5


@pytest.mark.parametrize('omega', [0.0, 0.3])
def test_screening_error_and_savings(omega):
    """Screened (1e-11) vs unscreened on 8 waters with a per-water localised
    density: |dK| and |1/4 tr(D dK)| <= 1e-8 and tasks skipped (reference
    tests/gpu/test_sgx_k.py:226-244, there on a converged water27 density)."""
    mol = waters(8, 7.0, 8)
    coords, weights = grid_subset(mol, 1, 20000, 5)
    dm = local_density(mol, seed=5)
    K0, s0 = _k_gpu(mol, coords, weights, dm, omega, tile_tol=0.0)
    K1, s1 = _k_gpu(mol, coords, weights, dm, omega, tile_tol=1e-11)
    assert s0['pairs_kept'] == s0['pairs_total']
    assert s1['pairs_kept'] < s1['pairs_total']
    # every skipped task is below 1e-11 per element; the synthetic density
    # (random within each water, diffuse functions fully weighted) sums them
    # to a few 1e-8 on single K elements, the energy stays below 1e-8
    assert np.max(np.abs(K1 - K0)) < 5e-8
    assert abs(0.25 * np.einsum('ij,ji->', dm, K1 - K0)) < 1e-8


def test_builder_api_and_out_of_scope():
    from pyscf_wb97mv_fast_gb300.gpu.sgx_k import (GpuKBuilder, SyntheticSGX,
                                                   Unsupported, get_k_only_gpu)
    from pyscf_wb97mv_fast_gb300.grids import build_grids
    mol = dimer('synthetic-svp')
    g = build_grids(mol, level=0)
    sgx = SyntheticSGX(mol, g)
    dm = density(mol.nao, 10, 7)
    b = GpuKBuilder(mol, tile_tol=0.0)
    K = get_k_only_gpu(b, sgx, dm)
    assert K.dtype == np.float64 and K.shape == (mol.nao, mol.nao)
    assert np.array_equal(K, K.T)
    Kref = oracle.cosx_k(mol, g.coords, g.weights, dm, 0.0)
    assert np.max(np.abs(K - Kref)) < 1e-6 * np.abs(Kref).max()
    assert b.last_stats['pairs_kept'] == b.last_stats['pairs_total']
    mol.omega = 0.3
    try:
        K3 = get_k_only_gpu(b, sgx, dm)
    finally:
        mol.omega = 0.0
    Kref3 = oracle.cosx_k(mol, g.coords, g.weights, dm, 0.3)
    assert np.max(np.abs(K3 - Kref3)) < 1e-6 * np.abs(Kref3).max()
    with pytest.raises(Unsupported):
        get_k_only_gpu(b, sgx, dm, hermi=0)
    with pytest.raises(Unsupported):
        get_k_only_gpu(b, sgx, np.stack([dm, 0.5 * dm]))
    asym = dm.copy()
    asym[0, 1] += 1e-3
    with pytest.raises(Unsupported):
        get_k_only_gpu(b, sgx, asym)


def test_multi_omega_build_matches_single_builds():
    """wb_cosx_get_k_multi shares AO values, F and the block statistics
    between the omegas: each of its matrices is bitwise the single-omega
    build; the builder's pending cache hands out the second omega for the
    same density and drops it for another one."""
    torch = _torch()
    from pyscf_wb97mv_fast_gb300.cosx import CosxEngine
    from pyscf_wb97mv_fast_gb300.gpu.sgx_k import GpuKBuilder, SyntheticSGX
    from pyscf_wb97mv_fast_gb300.grids import build_grids
    mol = waters(4, 6.0, 11)
    coords, weights = grid_subset(mol, 1, 9000, 5)
    dm = density(mol.nao, 12, 4)
    eng = CosxEngine(mol)
    c = eng.relative(coords)
    w = torch.as_tensor(weights, device=eng.device)
    qd = torch.as_tensor(dm, device=eng.device)
    oms = (0.0, 0.3, 0.11)
    Km = eng.get_k_multi(c, w, qd, oms, tile_tol=1e-11, tile_pts=4096)
    st_m = eng.last_stats
    kept = 0
    for j, om in enumerate(oms):
        Ks = eng.get_k(c, w, qd, om, tile_tol=1e-11, tile_pts=4096)
        kept += eng.last_stats['pairs_kept']
        assert torch.equal(Km[j], Ks), om
    assert st_m['pairs_kept'] == kept
    # the G-only entry point: one pass of the two-omega kernels per omega
    # pair, bitwise the single-omega G, the same tasks kept
    F = eng.ozaki_f(eng.ao_eval(c), qd)
    Gm = eng.g_multi(c, w, F, oms, 1e-11)
    kept_gm, kept_g = eng.last_stats['pairs_kept'], 0
    for j, om in enumerate(oms):
        Gs = eng.g(c, w, F, om, 1e-11)
        kept_g += eng.last_stats['pairs_kept']
        assert torch.equal(Gm[j], Gs), om
    assert kept_gm == kept_g
    # builder: omega 0 builds both, omega 0.3 comes from the pending set
    g = build_grids(mol, level=0)
    sgx = SyntheticSGX(mol, g)
    b = GpuKBuilder(mol, tile_tol=1e-11, omegas=(0.0, 0.3))
    b1 = GpuKBuilder(mol, tile_tol=1e-11)
    K0 = b.get_k(sgx, dm, 0.0)
    assert b.last_stats['from_multi'] is False
    K3 = b.get_k(sgx, dm, 0.3)
    assert b.last_stats['from_multi'] is True
    assert np.array_equal(K0, b1.get_k(sgx, dm, 0.0))
    assert np.array_equal(K3, b1.get_k(sgx, dm, 0.3))
    # a new density drops the pending set: no stale K
    dm2 = dm * 1.5
    b.get_k(sgx, dm2, 0.0)
    K3b = b.get_k(sgx, dm2, 0.3)
    assert b.last_stats['from_multi'] is True
    assert np.array_equal(K3b, b1.get_k(sgx, dm2, 0.3))
    b.get_k(sgx, dm2, 0.0)
    K3c = b.get_k(sgx, dm, 0.3)          # other density: built afresh
    assert b.last_stats['from_multi'] is False
    assert np.array_equal(K3c, K3)


def test_screening_error_dense_random_density():
    """A dense random density (F does not decay) is the hard case for the
    screen: the error stays below 1e-7 (K elements) and 1e-8 (energy)."""
    mol = waters(8, 7.0, 8)
    coords, weights = grid_subset(mol, 1, 20000, 5)
    dm = density(mol.nao, 40, 5)
    K0, _ = _k_gpu(mol, coords, weights, dm, 0.0, tile_tol=0.0)
    K1, s1 = _k_gpu(mol, coords, weights, dm, 0.0, tile_tol=1e-11)
    assert s1['pairs_kept'] < s1['pairs_total']
    assert np.max(np.abs(K1 - K0)) < 1e-7
    assert abs(0.25 * np.einsum('ij,ji->', dm, K1 - K0)) < 1e-8


@pytest.mark.parametrize('gemm', ['ozaki', 'emulated'])
@pytest.mark.parametrize('omega', [0.0, 0.3])
def test_gemm_modes_match_native_fp64(omega, gemm):
    """The Ozaki bf16 split (default) and cuBLAS FP64 emulation for
    F = X QD and K = X^T (w G) give the K of the native DGEMMs: the F
    roundings to FP32 agree except on rare ties (one ulp), so K agrees to
    FP32-noise level, far inside the oracle gate."""
    mol = waters(4, 5.0, 4)
    coords, weights = grid_subset(mol, 1, 30000, 2)
    dm = density(mol.nao, 20, 2)
    Kn, _ = _k_gpu(mol, coords, weights, dm, omega, gemm='native')
    Ke, st = _k_gpu(mol, coords, weights, dm, omega, gemm=gemm)
    assert np.max(np.abs(Ke - Kn)) < 1e-9 * np.abs(Kn).max()
    assert abs(0.25 * np.einsum('ij,ji->', dm, Ke - Kn)) < 1e-10


def test_ozaki_gemms_are_fp64_accurate():
    """The two Ozaki GEMMs alone against FP64 torch GEMMs on the same
    device operands: F bit-identical to fl32(X QD) on > 99 % of the
    entries and everywhere within the split's bound, nao 2^-38 times the
    row maximum of X and the column maximum of QD, plus the FP32 rounding;
    K = X^T (w G) to 1e-10 relative."""
    torch = _torch()
    from pyscf_wb97mv_fast_gb300.cosx import CosxEngine
    mol = waters(6, 6.0, 6)
    coords, weights = grid_subset(mol, 1, 40000, 3)
    dm = density(mol.nao, 30, 3)
    eng = CosxEngine(mol)
    c = eng.relative(coords)
    w = torch.as_tensor(weights, device=eng.device)
    qd = torch.as_tensor(dm, device=eng.device)
    X = eng.ao_eval(c)
    F_ref = (qd.T @ X).to(torch.float32)
    F_oz = eng.ozaki_f(X, qd)
    same = (F_oz == F_ref).double().mean().item()
    assert same > 0.99, same
    F64 = qd.T @ X
    rowmax = X.abs().max(dim=0).values                  # per point g
    colmax = qd.abs().max(dim=0).values                 # per AO mu
    bound = (2.0 ** -38 * mol.nao * colmax[:, None] * rowmax[None, :]
             + F64.abs() * 2.0 ** -24)
    assert bool(((F_oz.double() - F64).abs() <= bound).all())
    # K: the G of the real kernels on this grid, against FP64 torch, within
    # the split's bound: per 2048-point chunk c, 2^-40 Kc max_c|X_mu|
    # max_c|w G_nu| (42-bit digits relative to the chunk-column maxima)
    n = c.shape[0]
    G = eng.g(c, w, F_oz, 0.0, 0.0)
    K_oz = eng.ozaki_k(X, G, w)
    wpad = torch.nn.functional.pad(w, (0, X.shape[1] - n))
    wG = G.double() * wpad[None, :]
    K_ref = X @ wG.T
    kc = 2048
    ld = X.shape[1]
    nch = (ld + kc - 1) // kc
    pad = nch * kc - ld
    xm = torch.nn.functional.pad(X.abs(), (0, pad)).view(mol.nao, nch, kc).max(dim=2).values
    gm = torch.nn.functional.pad(wG.abs(), (0, pad)).view(mol.nao, nch, kc).max(dim=2).values
    bound = 2.0 ** -40 * kc * (xm @ gm.T)
    assert bool(((K_oz - K_ref).abs() <= bound).all())
    assert (K_oz - K_ref).abs().max().item() < 1e-10 * K_ref.abs().max().item()
