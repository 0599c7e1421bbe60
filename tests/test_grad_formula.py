"""The decomposition the GPU exchange gradient implements (wb_cosx_k_grad),
checked on the CPU with the FP64 oracle alone: for E = -1/4 tr(D K) at a
fixed grid,

  dE/dR_C = 1/2 sum_g w_g sum_{mu on C} grad X_g,mu (G D)_g,mu
            - 1/4 sum_g w_g F_g^T (dA^g/dR_C) F_g,

against Richardson-extrapolated central differences of the oracle energy
(the integral side differenced from the oracle's dense integrals).  Small
grid: the oracle's dense integrals hold (ng, nao, nao)."""
import numpy as np
import pytest

import oracle
from helpers import density, dimer, grid_subset


def _moved(mol, atom, axis, h):
    from pyscf_wb97mv_fast_gb300.basis import Molecule
    xyz = mol.atom_coords().copy()
    xyz[atom, axis] += h
    return Molecule(mol.symbols, xyz, mol.shells, mol.basis)


def _energy(mol, coords, weights, dm, omega):
    K = oracle.cosx_k(mol, coords, weights, dm, omega)
    return -0.25 * np.einsum('ij,ji->', dm, K)


@pytest.mark.parametrize('omega', [0.0, 0.3])
def test_gradient_decomposition_matches_energy_differences(omega):
    mol = dimer('synthetic-svp')
    coords, weights = grid_subset(mol, 1, 120, 31)
    dm = density(mol.nao, 10, 32)
    X = oracle.ao_eval(mol, coords)
    dX = oracle.ao_eval_deriv1(mol, coords)
    F = X @ dm
    H = oracle.cosx_g(mol, coords, F, omega) @ dm
    ao_atom = np.concatenate([[sh.atom] * sh.nao for sh in mol.shells])
    grad = np.zeros((mol.natm, 3))
    for x in range(3):
        v = 0.5 * np.einsum('g,gm,gm->m', weights, dX[1 + x], H)
        np.add.at(grad[:, x], ao_atom, v)
    h = 1e-5
    ref = np.zeros_like(grad)
    for a in range(mol.natm):
        for x in range(3):
            dA = (oracle.int3c1e(_moved(mol, a, x, h), coords, omega) -
                  oracle.int3c1e(_moved(mol, a, x, -h), coords, omega)) / (2 * h)
            grad[a, x] -= 0.25 * np.einsum('g,gi,gij,gj->', weights, F, dA, F)

            def central(step):
                return (_energy(_moved(mol, a, x, step), coords, weights, dm, omega) -
                        _energy(_moved(mol, a, x, -step), coords, weights, dm, omega)
                        ) / (2 * step)
            ref[a, x] = (4.0 * central(5e-5) - central(1e-4)) / 3.0
    assert np.abs(grad - ref).max() < 1e-8 * np.abs(ref).max() + 1e-11
