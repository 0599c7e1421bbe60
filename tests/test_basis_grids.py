"""Synthetic molecules, basis conventions and grids (CPU)."""
import math

import numpy as np
import pytest

from pyscf_wb97mv_fast_gb300.basis import (Molecule, cart2sph, cart_components,
                                           gto_norm)
from pyscf_wb97mv_fast_gb300.grids import angular_grid, build_grids, radial_grid
from pyscf_wb97mv_fast_gb300.systems import alkane, drug_like, water_cluster


def test_cart2sph_orthonormal_on_the_sphere():
    xyz, w = angular_grid(20)
    for l in range(4):
        P = np.stack([xyz[:, 0] ** i * xyz[:, 1] ** j * xyz[:, 2] ** k
                      for (i, j, k) in cart_components(l)], axis=1)
        S = P @ cart2sph(l)
        G = (S * w[:, None]).T @ S
        assert np.allclose(G, np.eye(2 * l + 1), atol=1e-12)


def _real_harmonic_table(l, x, y, z):
    """The real spherical harmonics r^l Y_lm in Cartesian form, unit-
    normalised on the sphere, written out from the standard table (not from
    the solid-harmonic expansion that ``cart2sph`` evaluates), in the
    column order of PySCF's ``gto.mole.cart2sph(l)`` that the reference
    applies (``gpu/ao_eval.py:73``, ``gpu/shellpairs.py:219``): (x, y, z)
    for l = 1, m = -l .. l for l >= 2."""
    pi = math.pi
    if l == 0:
        return [np.full_like(x, 0.5 / math.sqrt(pi))]
    if l == 1:
        c = math.sqrt(3.0 / (4.0 * pi))
        return [c * x, c * y, c * z]
    if l == 2:
        a = 0.5 * math.sqrt(15.0 / pi)
        return [a * x * y, a * y * z,
                0.25 * math.sqrt(5.0 / pi) * (2 * z * z - x * x - y * y),
                a * x * z, 0.25 * math.sqrt(15.0 / pi) * (x * x - y * y)]
    if l == 3:
        c3 = 0.25 * math.sqrt(35.0 / (2.0 * pi))
        c1 = 0.25 * math.sqrt(21.0 / (2.0 * pi))
        return [c3 * y * (3 * x * x - y * y),
                0.5 * math.sqrt(105.0 / pi) * x * y * z,
                c1 * y * (4 * z * z - x * x - y * y),
                0.25 * math.sqrt(7.0 / pi) * z * (2 * z * z - 3 * x * x - 3 * y * y),
                c1 * x * (4 * z * z - x * x - y * y),
                0.25 * math.sqrt(105.0 / pi) * z * (x * x - y * y),
                c3 * x * (x * x - 3 * y * y)]
    raise ValueError(l)


@pytest.mark.parametrize('l', [0, 1, 2, 3])
def test_cart2sph_matches_the_real_harmonic_table(l):
    """Order, signs and normalisation of every spherical component against
    an independent statement of the convention: a column permutation, a sign
    flip or a wrong m normalisation would pass the orthonormality test above
    but fails here."""
    rng = np.random.default_rng(l)
    x, y, z = rng.uniform(-1.5, 1.5, size=(3, 64))
    P = np.stack([x ** i * y ** j * z ** k for (i, j, k) in cart_components(l)],
                 axis=1)
    got = P @ cart2sph(l)
    want = np.stack(_real_harmonic_table(l, x, y, z), axis=1)
    np.testing.assert_allclose(got, want, rtol=0, atol=1e-13)


@pytest.mark.parametrize('basis', ['synthetic-svp', 'synthetic-tzvp'])
def test_contracted_functions_are_normalised(basis):
    atoms = water_cluster(1, 1.0, seed=0) + [('F', (3.0, 0, 0)), ('S', (6.0, 0, 0)),
                                             ('Cl', (9.0, 0, 0)), ('C', (12.0, 0, 0)),
                                             ('N', (15.0, 0, 0))]
    mol = Molecule.build(atoms, basis)
    r, w = radial_grid(400, 1.0)
    for sh in mol.shells:
        for c in range(sh.nctr):
            rad = (sh.coeffs[:, c][None, :] * r[:, None] ** sh.l
                   * np.exp(-np.outer(r ** 2, sh.exps))).sum(axis=1)
            assert (rad ** 2 * w).sum() == pytest.approx(1.0, rel=1e-6)


def test_water_cluster_geometry():
    atoms = water_cluster(27, box=10.0, seed=27)
    xyz = np.array([a[1] for a in atoms]).reshape(27, 3, 3)
    o = xyz[:, 0]
    d = np.linalg.norm(o[:, None] - o[None], axis=2) + np.eye(27) * 99
    assert d.min() >= 2.7
    assert np.all((o >= 0) & (o <= 10.0))
    for w in xyz:
        oh1, oh2 = w[1] - w[0], w[2] - w[0]
        assert np.linalg.norm(oh1) == pytest.approx(0.9572)
        ang = math.degrees(math.acos(oh1 @ oh2 / (np.linalg.norm(oh1) * np.linalg.norm(oh2))))
        assert ang == pytest.approx(104.52)
    assert water_cluster(27, 10.0, 27) == atoms          # seeded


def test_alkane_geometry_and_basis_size():
    atoms = alkane(20)
    assert len(atoms) == 62
    xyz = np.array([a[1] for a in atoms])
    sym = [a[0] for a in atoms]
    d = np.linalg.norm(xyz[:, None] - xyz[None], axis=2) + np.eye(62) * 99
    for i, s in enumerate(sym):
        nb = np.sort(d[i][d[i] < 1.6])
        if s == 'C':
            assert len(nb) == 4
            assert np.allclose(nb[nb > 1.3], 1.53) and np.allclose(nb[nb < 1.3], 1.09)
    assert Molecule.build(atoms, 'synthetic-tzvp').nao == 872
    assert Molecule.build(water_cluster(27, 10.0, 27)).nao == 648


def test_grid_integrates_gaussians():
    mol = Molecule.build(water_cluster(2, 3.2, seed=1))
    g = build_grids(mol, level=1)
    for a in (0.5, 3.0):
        c = mol.atom_coords()[1]
        f = np.exp(-a * ((g.coords - c) ** 2).sum(axis=1))
        assert (f * g.weights).sum() == pytest.approx((math.pi / a) ** 1.5, rel=1e-3)


def test_grid_subblocks_are_compact():
    mol = Molecule.build(water_cluster(8, 7.0, seed=8))
    g = build_grids(mol, level=1)
    n = g.size // 32 * 32
    blocks = g.coords[:n].reshape(-1, 32, 3)
    cen = blocks.mean(axis=1)
    rad = np.linalg.norm(blocks - cen[:, None], axis=2).max(axis=1)
    assert np.median(rad) < 1.0          # bohr


def test_gto_norm():
    for l in range(4):
        a = 1.7
        r, w = radial_grid(300, 1.0)
        v = (gto_norm(l, a) * r ** l * np.exp(-a * r * r)) ** 2
        assert (v * w).sum() == pytest.approx(1.0, rel=1e-8)


def test_drug_like_molecule():
    """Seeded; the drug elements present; bonded distances only between
    bonded atoms; SVP / TZVP sizes (f shells on the heavy atoms)."""
    atoms = drug_like(0)
    assert drug_like(0) == atoms
    sym = [a[0] for a in atoms]
    for x in ('C', 'N', 'O', 'S', 'F', 'Cl', 'H'):
        assert x in sym
    xyz = np.array([a[1] for a in atoms])
    d = np.linalg.norm(xyz[:, None] - xyz[None], axis=2) + np.eye(len(sym)) * 99
    assert d.min() > 0.9
    heavy = [i for i, s in enumerate(sym) if s != 'H']
    dh = d[np.ix_(heavy, heavy)]
    assert dh.min() > 1.3
    svp = Molecule.build(atoms, 'synthetic-svp')
    tz = Molecule.build(atoms, 'synthetic-tzvp')
    assert tz.nao > 1.9 * svp.nao
    assert max(sh.l for sh in tz.shells) == 3


def test_oracle_partition_gives_the_native_grid():
    """The reference arm of the bench builds its grid with the oracle's
    Becke partition (no product library); the grid is the native one."""
    import oracle
    from pyscf_wb97mv_fast_gb300.basis import Molecule
    from pyscf_wb97mv_fast_gb300.grids import build_grids
    from pyscf_wb97mv_fast_gb300.systems import water_cluster
    mol = Molecule.build(water_cluster(4, box=6.0, seed=3), 'synthetic-svp')
    a = build_grids(mol, level=0)
    b = build_grids(mol, level=0, partition=oracle.becke_partition)
    np.testing.assert_array_equal(a.coords, b.coords)
    np.testing.assert_allclose(a.weights, b.weights, rtol=1e-14, atol=0)


def test_read_xyz_and_drug_fixture():
    from pyscf_wb97mv_fast_gb300.systems import read_xyz
    atoms = read_xyz('3\ncomment\nO 0 0 0\nh 0.9572 0 0\nH -0.24 0.927 0\n')
    assert [a[0] for a in atoms] == ['O', 'H', 'H']
    assert atoms[1][1] == (0.9572, 0.0, 0.0)
    with pytest.raises(ValueError):
        read_xyz('4\nc\nO 0 0 0\n')
    from helpers import DRUGS, drug
    sizes = {n: drug(n).nao for n in DRUGS}
    assert all(400 < v < 900 for v in sizes.values()), sizes
    # Br carries d shells in both structures and an f shell in TZVP
    m = drug('bromazepam')
    assert 'Br' in m.symbols
    assert max(sh.l for sh in m.shells if m.symbols[sh.atom] == 'Br') == 3
