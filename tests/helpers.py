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


class ToyFunctional:
    """Stand-in XcFunctional (libxc convention) for the semilocal flow tests,
    PySCF's libxc being absent:  e(rho, sigma, tau) = -Cx rho^(4/3)
    + a sigma exp(-rho) + b tau rho / (1 + rho), exc = e / rho, and
    vrho, vsigma, vtau its partial derivatives; a = b = 0 for LDA (no
    vsigma, vtau), b = 0 for GGA (no vtau).  Points with rho < 1e-12 give
    zeros, like libxc's density threshold."""

    CX = 0.7385587663820224

    def __init__(self, xctype='MGGA', a=0.05, b=0.2):
        self.xctype = xctype
        self.a = a if xctype in ('GGA', 'MGGA') else 0.0
        self.b = b if xctype == 'MGGA' else 0.0

    def eval(self, rho):
        rho = np.asarray(rho, dtype=np.float64)
        r = rho[0]
        ok = r >= 1e-12
        rr = np.where(ok, r, 1.0)
        sigma = (rho[1:4] ** 2).sum(axis=0)
        tau = rho[4]
        ex = np.exp(-rr)
        e = -self.CX * rr ** (4.0 / 3.0) + self.a * sigma * ex + self.b * tau * rr / (1.0 + rr)
        vrho = (-4.0 / 3.0 * self.CX * rr ** (1.0 / 3.0) - self.a * sigma * ex
                + self.b * tau / (1.0 + rr) ** 2)
        exc = np.where(ok, e / rr, 0.0)
        vrho = np.where(ok, vrho, 0.0)
        vsigma = np.where(ok, self.a * ex, 0.0) if self.xctype != 'LDA' else None
        vtau = np.where(ok, self.b * rr / (1.0 + rr), 0.0) if self.xctype == 'MGGA' else None
        return exc, vrho, vsigma, vtau


class ToyNumInt:
    """The two NumInt pieces the flow reads: the xc type."""

    def __init__(self, xctype):
        self.xctype = xctype

    def _xc_type(self, xc_code):
        return self.xctype


DRUGS = ('bromazepam', 'caffeine', 'chlorpromazine', 'fluoxetine', 'ibuprofen',
         'sulfamethoxazole')


def drug(name, basis='synthetic-tzvp'):
    """One of the reference's six validation molecules
    (benchmarks/systems/drugs/*.xyz), from tests/golden/drugs.npz."""
    import os
    d = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)),
                             'golden', 'drugs.npz'))
    atoms = [(s, tuple(float(x) for x in c))
             for s, c in zip(d[name + '_symbols'].tolist(), d[name + '_coords'])]
    return Molecule.build(atoms, basis)
