"""The FP64 oracle against the reference's own outputs (tests/golden/,
made by tests/golden/make_golden.py from the reference's Python) and
closed forms.  CPU only."""
import os

import numpy as np
import pytest

import oracle
from helpers import dimer

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), 'golden')


def _load(name):
    return np.load(os.path.join(GOLDEN, name))


def test_boys_matches_reference_boys_ref():
    d = _load('boys.npz')
    for k, t in enumerate(d['boys_T']):
        f = oracle.boys(6, float(t))
        ref = d['boys_ref'][:, k]
        assert np.max(np.abs(f - ref) / ref) < 5e-13, t


def test_boys_closed_forms():
    for n in range(13):
        assert oracle.boys(12, 0.0)[n] == pytest.approx(1.0 / (2 * n + 1), rel=1e-15)
    t = 3.7
    # F_0(t) = sqrt(pi/t)/2 erf(sqrt t)
    from math import erf, pi, sqrt
    assert oracle.boys(0, t)[0] == pytest.approx(0.5 * sqrt(pi / t) * erf(sqrt(t)),
                                                 rel=1e-14)


def test_native_boys_table_matches_reference_table():
    """The FP32 Taylor-table entries F_n(T_k) hi / lo of this library equal
    the reference's (gpu/boys.py _build_table, j = 0 column) to 1 ulp."""
    from pyscf_wb97mv_fast_gb300.cosx import boys_f64_host
    d = _load('boys.npz')
    hi_ref, lo_ref = d['boys_table_hi'], d['boys_table_c0lo']
    nodes = hi_ref.shape[0]
    mism = 0
    for k in range(nodes):
        f = boys_f64_host(12, 0.25 * k)
        hi = f[:7].astype(np.float32)
        lo = (f[:7] - hi.astype(np.float64)).astype(np.float32)
        diff = np.abs(hi.view(np.int32) - hi_ref[k, :, 0].view(np.int32))
        assert diff.max() <= 1, k
        mism += int((diff != 0).sum())
        # the remainder carries the FP64 value to ~1e-15 relative
        assert np.allclose(hi.astype(np.float64) + lo,
                           hi_ref[k, :, 0].astype(np.float64) + lo_ref[k],
                           rtol=1e-13, atol=0)
    assert mism <= 0.01 * nodes * 7


@pytest.mark.parametrize('tag,basis,gen', [('svp', 'synthetic-svp', False),
                                           ('tzvp', 'synthetic-tzvp', False),
                                           ('gen', 'synthetic-svp', True)])
@pytest.mark.parametrize('omega', [0.0, 0.3])
def test_int3c1e_matches_reference(tag, basis, gen, omega):
    d = _load('int3c1e_%s.npz' % tag)
    mol = dimer(basis, gen)
    A = oracle.int3c1e(mol, d['coords'], omega)
    ref = d['A_w%g' % omega]
    assert np.max(np.abs(A - ref)) < 1e-12 * max(1.0, np.abs(ref).max())


@pytest.mark.parametrize('tag,basis,gen', [('svp', 'synthetic-svp', False),
                                           ('tzvp', 'synthetic-tzvp', False),
                                           ('gen', 'synthetic-svp', True)])
def test_ao_eval_matches_reference(tag, basis, gen):
    d = _load('int3c1e_%s.npz' % tag)
    X = oracle.ao_eval(dimer(basis, gen), d['ao_coords'])
    assert np.max(np.abs(X - d['ao'])) < 1e-13 * np.abs(d['ao']).max()


@pytest.mark.parametrize('omega', [0.0, 0.3])
def test_k_matches_reference(omega):
    d = _load('k_svp.npz')
    K = oracle.cosx_k(dimer(), d['coords'], d['weights'], d['dm'], omega)
    ref = d['K_w%g' % omega]
    assert np.max(np.abs(K - ref)) < 1e-12 * np.abs(ref).max()


def test_cosx_g_is_the_dense_contraction():
    d = _load('int3c1e_svp.npz')
    mol = dimer()
    F = np.random.default_rng(0).normal(size=(len(d['coords']), mol.nao))
    G = oracle.cosx_g(mol, d['coords'], F, 0.3)
    ref = np.einsum('gmn,gm->gn', d['A_w0.3'], F)
    assert np.max(np.abs(G - ref)) < 1e-12 * np.abs(ref).max()


def test_bound_is_an_upper_bound_of_reference_integrals():
    """The reference's pair_bound (golden) bounds |A| of the oracle's own
    integrals on each block (reference tests/gpu/test_shellpairs.py:39-56)."""
    d = _load('int3c1e_svp.npz')
    mol = dimer()
    rows = d['pair_rows']
    ao = mol.ao_loc_nr()
    for k in range(3):
        blk = d['bound_block%d' % k]
        A = oracle.int3c1e(mol, blk, 0.0)
        b = d['bound%d' % k]
        for p, r in enumerate(rows):
            i0, j0, ish, jsh = int(r[0]), int(r[1]), int(r[2]), int(r[3])
            ni = ao[ish + 1] - ao[ish]
            nj = ao[jsh + 1] - ao[jsh]
            assert np.abs(A[:, i0:i0 + ni, j0:j0 + nj]).max() <= b[p] * (1 + 1e-12)


def test_vv10_matches_reference_kernel_sum():
    """Reference NumPy kernel_sum (FP32 pairs, Kahan tiles) vs the FP64
    brute force: relative 1e-6 (reference gate tests/gpu/test_xc_vv10.py:
    275-293) on the cluster near the origin; the far cluster (x ~ 30 bohr)
    carries the FP32 rounding of its coordinates (a few 1e-6)."""
    d = _load('vv10.npz')
    F, U, W = oracle.vv10_sum(d['xyz'], d['q'], d['w0'], d['kappa'])
    for got, ref in ((F, d['F']), (U, d['U']), (W, d['W'])):
        rel = np.abs(got - ref) / np.abs(ref)
        assert rel[:500].max() < 1e-6
        assert rel.max() < 1e-5


@pytest.mark.parametrize('tag,basis,gen', [('svp', 'synthetic-svp', False),
                                           ('tzvp', 'synthetic-tzvp', False),
                                           ('gen', 'synthetic-svp', True)])
def test_ao_deriv1_matches_reference(tag, basis, gen):
    d = _load('int3c1e_%s.npz' % tag)
    X = oracle.ao_eval_deriv1(dimer(basis, gen), d['ao_coords'])
    assert np.max(np.abs(X - d['ao1'])) < 1e-13 * np.abs(d['ao1']).max()


def test_vv10_flow_matches_reference():
    """The oracle's FP64 VV10 flow vs the reference's gpu_nr_nlc_vxc run on
    its NumPy backend (FP64 AO and GEMMs, FP32 pair sum)."""
    d = _load('vv10_flow.npz')
    n, e, v = oracle.nlc_vxc(dimer(), d['coords'], d['weights'], d['dm'],
                             [((float(d['nlc_b']), float(d['nlc_c'])), 1.0)])
    assert abs(n - d['nelec']) < 1e-12
    assert abs(e - d['exc']) < 1e-9
    assert np.max(np.abs(v - d['vmat'])) < 1e-9
