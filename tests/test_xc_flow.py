"""Semilocal XC flow (NumInt.nr_rks) on the CPU: the FP64 oracle restatement
and the host chain rule (reference tests: tests/gpu/test_xc_vv10.py:50-86).

PySCF's nr_rks and libxc are absent, so the oracle flow is pinned by a
property instead: the potential matrix is the derivative of the XC energy,
tr(vmat P) = d E_xc(D + h P) / dh at h = 0 for symmetric P (central
difference), which checks the chain rule, the factor 1/2 conventions and the
tau term together.  The AO values it uses are pinned to the reference's AO
evaluator by the golden vectors."""
import numpy as np
import pytest

import oracle
from helpers import ToyFunctional, dimer, density, grid_subset

from pyscf_wb97mv_fast_gb300.gpu.xc import chain_rule


@pytest.mark.parametrize('xctype', ['LDA', 'GGA', 'MGGA'])
def test_oracle_flow_potential_is_the_energy_derivative(xctype):
    mol = dimer()
    coords, weights = grid_subset(mol, 1, 3000, 2)
    ao = oracle.ao_eval_deriv1(mol, coords)
    dm = density(mol.nao, 5, 1)
    fn = ToyFunctional(xctype)
    n0, e0, v0 = oracle.nr_rks(mol, coords, weights, dm, fn, xctype, ao=ao)
    assert np.allclose(v0, v0.T, rtol=0, atol=1e-14 * np.abs(v0).max())
    rng = np.random.default_rng(3)
    P = rng.normal(size=dm.shape)
    P = 0.5 * (P + P.T)
    # central difference: truncation ~ h^2 (3.5e-9 at h = 1e-5 here)
    h = 1e-5
    ep = oracle.nr_rks(mol, coords, weights, dm + h * P, fn, xctype, ao=ao)[1]
    em = oracle.nr_rks(mol, coords, weights, dm - h * P, fn, xctype, ao=ao)[1]
    fd = (ep - em) / (2 * h)
    an = float(np.sum(v0 * P))
    assert abs(fd - an) <= 1e-7 * max(1.0, abs(an)), (fd, an)
    assert n0 > 0


def test_chain_rule_matches_the_oracle_restatement():
    rng = np.random.default_rng(0)
    rho = rng.normal(size=(5, 37))
    exc, vrho, vsigma, vtau = (rng.normal(size=37) for _ in range(4))
    for vs, vt in ((vsigma, vtau), (vsigma, None), (None, None)):
        e1, v1 = chain_rule(rho, exc, vrho, vs, vt)
        e2, v2 = oracle.xc_chain_rule(rho, exc, vrho, vs, vt)
        assert np.array_equal(e1, e2) and np.array_equal(v1, v2)
    _, v = chain_rule(rho, exc, vrho, vsigma, None)
    assert np.array_equal(v[1:4], 2.0 * vsigma * rho[1:4]) and not v[4].any()
