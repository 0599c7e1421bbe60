"""Shared test inputs: synthetic molecules, grids, density matrices."""
import numpy as np

from pyscf_wb97mv_fast_gb300.basis import Molecule
from pyscf_wb97mv_fast_gb300.grids import build_grids
from pyscf_wb97mv_fast_gb300.systems import water_cluster, water_dimer


def dimer(basis='synthetic-svp', gen_contract=False):
    return Molecule.build(water_dimer(), basis, gen_contract=gen_contract)


def waters(n, box, seed, basis='synthetic-svp'):
    return Molecule.build(water_cluster(n, box=box, seed=seed), basis)


def density(nao, nocc, seed=0):
    """D = 2 C C^T with C (nao, nocc) seeded N(0, 1), orthonormalised by QR."""
    rng = np.random.default_rng(seed)
    c, _ = np.linalg.qr(rng.normal(size=(nao, nocc)))
    return 2.0 * c @ c.T


def grid_subset(mol, level, n, seed=0):
    g = build_grids(mol, level=level)
    if n is None or n >= g.size:
        return g.coords, g.weights
    rng = np.random.default_rng(seed)
    sel = np.sort(rng.choice(g.size, n, replace=False))
    return g.coords[sel], g.weights[sel]


def local_density(mol, atoms_per_unit=3, nocc_per_unit=5, seed=0):
    """D = 2 C C^T with every occupied orbital a random orthonormal mix of
    the AOs of one molecular unit (e.g. one water): a density that decays
    between units the way a real cluster density does."""
    rng = np.random.default_rng(seed)
    ao = mol.ao_loc_nr()
    units = {}
    for s, sh in enumerate(mol.shells):
        units.setdefault(sh.atom // atoms_per_unit, []).extend(range(ao[s], ao[s + 1]))
    cols = []
    for u in sorted(units):
        idx = np.array(units[u])
        q, _ = np.linalg.qr(rng.normal(size=(len(idx), nocc_per_unit)))
        c = np.zeros((mol.nao, nocc_per_unit))
        c[idx] = q
        cols.append(c)
    c = np.hstack(cols)
    return 2.0 * c @ c.T
