"""ScfRun, the SCF loop of DeviceRKS.kernel cut at its Fock builds (the
unit BatchedRKS steps many of), driven on the CPU with a stand-in
molecule: a 2x2 model Fock operator whose energy converges geometrically,
so the stage plan, the incremental-base bookkeeping and the convergence
test run without a GPU."""
import math

import pytest

torch = pytest.importorskip('torch')

from pyscf_wb97mv_fast_gb300.scf import ScfRun  # noqa: E402


class _Stand:
    """The members of DeviceRKS that ScfRun uses."""
    device = torch.device('cpu')
    verbose = False
    t_setup = 0.0

    def __init__(self):
        self.builds = []

    def core_guess(self):
        return torch.eye(2, dtype=torch.float64)

    def _stage_grids(self, stage):
        return {'stage': stage}

    def gemm_mode(self, fp64, inc32):
        return 'fp32' if not fp64 else ('split64' if inc32 else 'fp64')

    def _commutator(self, F, D):
        return F - D

    def _diag(self, F):
        return F, None


def _drive(run, rks, rate=0.3):
    """Fock builds whose energy error and gradient shrink by `rate` a
    cycle (the FP32 stages stall at 1e-7, the FP64 ones go on)."""
    err = 1.0
    while not run.done:
        req = run.request()
        rks.builds.append((req['grids']['stage'], req['fp64'], req['base'] is not None,
                           req['k_mode'], req['gemm']))
        floor = 0.0 if req['fp64'] else 1e-7
        err = max(err * rate, floor)
        E = torch.tensor(-1.0 + err, dtype=torch.float64)
        F = run.D + err * torch.eye(2, dtype=torch.float64) / math.sqrt(2.0)
        base = req['base'] if req['base'] is not None else {'D': run.D}
        run.advance(E, F, {}, base)
    return run.result()


def test_staged_run_switches_stages_and_keeps_one_fp64_base():
    rks = _Stand()
    out = _drive(ScfRun(rks, 'mixed', conv_tol=1e-9, conv_tol_grad=1e-5), rks)
    assert out['converged']
    stages = [b[0] for b in rks.builds]
    assert stages[0] == 0 and 2 in stages
    assert stages == sorted(stages)                    # no stage goes back
    fp64 = [b for b in rks.builds if b[1]]
    assert fp64, 'the FP64 tail ran'
    # the tail: one full FP64 build, then increments on it (no periodic
    # rebuild), exchange increments on the FP32 kernels, quadrature GEMMs
    # through the FP64 split
    assert not fp64[0][2] and all(b[2] for b in fp64[1:])
    assert fp64[0][3] == 'fp64' and all(b[3] == 'fp32' for b in fp64[1:])
    assert all(b[4] == 'split64' for b in fp64)
    # the FP32 stages build in full on the FP32 kernels
    assert all(not b[2] and b[3] == 'fp32' and b[4] == 'fp32'
               for b in rks.builds if not b[1])
    assert [s['stage'] for s in out['stages']][:2] == [0, 1]


def test_fp64_run_rebuilds_every_eight_cycles():
    rks = _Stand()
    out = _drive(ScfRun(rks, 'fp64', conv_tol=1e-30, conv_tol_grad=1e-30,
                        max_cycle=20), rks, rate=0.9)
    assert out['cycles'] == 20 and not out['converged']
    full = [i for i, b in enumerate(rks.builds) if not b[2]]
    assert full == [0, 8, 16]
    assert all(b[3] == 'fp64' and b[4] == 'fp64' for b in rks.builds)


def test_reference_energy_and_bad_precision():
    rks = _Stand()
    out = _drive(ScfRun(rks, 'fp64', reference_energy=-1.0), rks)
    assert out['converged'] and abs(out['error_vs_reference']) < 1e-9
    assert all('err' in h for h in out['history'])
    with pytest.raises(ValueError):
        ScfRun(rks, 'bf16')
    assert ScfRun(rks, 'mixed', max_cycle=0).done
