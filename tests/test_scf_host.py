"""Host-side pieces of the device SCF (CPU): the functional against the
oracle's independent restatement and against finite differences, the
DIIS extrapolation, and the staging plan it drives."""
import math

import numpy as np
import pytest


def test_functional_matches_oracle_restatement():
    import torch
    from oracle.scf import Functional
    from pyscf_wb97mv_fast_gb300.scf import RshLdaVv10
    rho = np.concatenate([np.geomspace(1e-13, 1e4, 3000), [0.0, 1e-15]])
    e, v = RshLdaVv10().eval(torch.as_tensor(rho))
    eo, vo = Functional().eval(rho)
    np.testing.assert_allclose(e.numpy(), eo, rtol=1e-12, atol=1e-300)
    np.testing.assert_allclose(v.numpy(), vo, rtol=1e-11, atol=1e-300)


def test_functional_potential_is_the_energy_derivative():
    import torch
    from pyscf_wb97mv_fast_gb300.scf import RshLdaVv10
    f = RshLdaVv10()
    rho = torch.as_tensor(np.geomspace(1e-9, 1e3, 800))
    _, v = f.eval(rho)
    h = rho * 1e-5
    fd = (f.eval(rho + h)[0] - f.eval(rho - h)[0]) / (2 * h)
    assert float(((fd - v).abs() / v.abs()).max()) < 1e-7


def test_sr_attenuation_limits_and_branch_continuity():
    import torch
    from pyscf_wb97mv_fast_gb300.scf import _sr_attenuation
    eps = 1e-9
    a = torch.as_tensor([1e-6, 1.5 - eps, 1.5, 1.5 + eps, 1e3], dtype=torch.float64)
    F, dF = _sr_attenuation(a)
    assert abs(float(F[0]) - 1.0) < 1e-5             # no attenuation at high density
    # the closed form (below 1.5) meets the series (above): the jump is the
    # slope across 2 eps, to 1e-13
    assert abs(float(F[1] - F[3]) + 2 * eps * float(dF[2])) < 1e-13
    assert abs(float(dF[1] - dF[3])) < 1e-9
    assert abs(float(F[4]) * 36e6 - 1.0) < 1e-6       # F -> 1 / (36 a^2)
    # against 40-digit values of the closed form (mpmath)
    ref = {1.0: 0.026772142179266237, 1.5: 0.012143137310041640, 3.0: 0.0030736105196919338}
    got = _sr_attenuation(torch.as_tensor(list(ref), dtype=torch.float64))[0]
    for (k, v), g in zip(ref.items(), got):
        assert abs(float(g) / v - 1.0) < 1e-12, k


def test_cdiis_extrapolates_a_linear_fixed_point():
    """On F(D) linear and e = F - F*, DIIS with two vectors lands on F*."""
    import torch
    from pyscf_wb97mv_fast_gb300.scf import _Cdiis
    rng = np.random.default_rng(0)
    Fstar = torch.as_tensor(rng.normal(size=(5, 5)))
    R = torch.as_tensor(rng.normal(size=(5, 5)))
    d = _Cdiis(8)
    for t in (1.0, 0.3):              # errors along one direction: solvable
        Fk = Fstar + t * R
        out = d.update(Fk, Fk - Fstar)
    assert float((out - Fstar).abs().max()) < 1e-10
    assert d.update(Fstar, Fstar - Fstar) is not None


def test_stage_plan_reaches_the_fp64_tail():
    from pyscf_wb97mv_fast_gb300.staging.schedule import StagePlan
    p = StagePlan(fp64_final=True, tau_fp64=1e-6, tau_fp64_g=1e-4)
    assert p.after_cycle(math.inf, 1e-1) is None
    assert p.after_cycle(1e-2, 1e-4)[0:2] == ('stage', 1)
    assert p.after_cycle(1e-7, 1e-4)[0:2] == ('stage', 2)
    assert not p.may_converge
    assert p.after_cycle(1e-7, 1e-5) == ('fp64', False)
    assert p.may_converge
