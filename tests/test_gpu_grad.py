"""COSX exchange nuclear gradient (wb_cosx_k_grad, grid response off)
against central finite differences of the FP64 oracle's energy
E = -1/4 tr(D K) with the basis centres moved and the grid held fixed.
The reference has no GPU gradient; it uses stock PySCF's SGX gradient with
the grid response off (README.md:134-137, :168)."""
import numpy as np
import pytest

import oracle
from helpers import density, dimer, grid_subset

pytestmark = pytest.mark.gpu


def _moved(mol, atom, axis, h):
    from pyscf_wb97mv_fast_gb300.basis import Molecule
    xyz = mol.atom_coords().copy()
    xyz[atom, axis] += h
    return Molecule(mol.symbols, xyz, mol.shells, mol.basis)


def _fd_grad(mol, coords, weights, dm, omega, h=5e-5):
    """Central differences at h and 2h, Richardson-extrapolated (grid
    points near the nuclei give the energy large high derivatives: the plain
    central difference at h = 1e-4 is off by ~1e-7, the extrapolation from
    1e-4 / 2e-4 by ~4e-9 with TZVP; from 5e-5 / 1e-4 by ~2e-10)."""
    def central(step):
        g = np.zeros((mol.natm, 3))
        for a in range(mol.natm):
            for x in range(3):
                e = []
                for s in (1, -1):
                    K = oracle.cosx_k(_moved(mol, a, x, s * step), coords, weights,
                                      dm, omega)
                    e.append(-0.25 * np.einsum('ij,ji->', dm, K))
                g[a, x] = (e[0] - e[1]) / (2 * step)
        return g
    return (4.0 * central(h) - central(2 * h)) / 3.0


@pytest.mark.parametrize('basis,gen,npts', [('synthetic-svp', False, 1500),
                                            ('synthetic-tzvp', False, 600),
                                            ('synthetic-svp', True, 1000)])
@pytest.mark.parametrize('omega', [0.0, 0.3])
def test_k_gradient_matches_finite_differences(basis, gen, npts, omega):
    import torch
    from pyscf_wb97mv_fast_gb300.cosx import CosxEngine
    mol = dimer(basis, gen)
    coords, weights = grid_subset(mol, 1, npts, 21)
    dm = density(mol.nao, 10, 22)
    eng = CosxEngine(mol)
    c = eng.relative(coords)
    w = torch.as_tensor(weights, device=eng.device)
    g = eng.k_grad(c, w, dm, omega)
    ref = _fd_grad(mol, coords, weights, dm, omega)
    err = np.abs(g - ref).max()
    assert err < 1e-7 * np.abs(ref).max() + 1e-10, (err, np.abs(ref).max())
    assert np.array_equal(g, eng.k_grad(c, w, dm, omega))      # reproducible


def test_k_gradient_screened():
    """tile_tol = 1e-11 drops tasks; the gradient moves by far less than
    the gradient gates of the reference's validation (1e-5 Ha/bohr)."""
    import torch
    from pyscf_wb97mv_fast_gb300.cosx import CosxEngine
    from helpers import local_density, waters
    mol = waters(4, 6.0, 23)
    coords, weights = grid_subset(mol, 1, 6000, 24)
    dm = local_density(mol, seed=25)
    eng = CosxEngine(mol)
    c = eng.relative(coords)
    w = torch.as_tensor(weights, device=eng.device)
    g0 = eng.k_grad(c, w, dm, 0.0, tile_tol=0.0)
    g1 = eng.k_grad(c, w, dm, 0.0, tile_tol=1e-11)
    assert np.abs(g1 - g0).max() < 1e-7
