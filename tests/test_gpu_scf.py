"""The device SCF against the oracle's host SCF (oracle/scf.py): the same
functional, grids and algorithm, FP64 and unscreened on the host.

* the plain FP64 device form reaches the oracle's energy to 1e-9 Ha (its
  screens, k_tile_tol 1e-11 and the Hartree screen, are the difference);
* the mixed-precision staged form (FP32 stages on coarse then final
  grids, FP64 tail) reaches it to 1e-8 Ha, the energy tolerance of the staged path;
* the per-cycle pieces match the oracle's Fock build on a fixed density.

The oracle energies come from tests/golden/scf_energies.json (written by
tests/golden/make_scf_golden.py, which runs oracle/scf.py): the water dimer
and eight seeded waters in SVP, and ethane in TZVP (f shells).
"""
import json
import os

import numpy as np
import pytest

from helpers import dimer

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))


def _golden():
    with open(os.path.join(HERE, 'golden', 'scf_energies.json')) as fh:
        return json.load(fh)


def _dimer_case():
    from pyscf_wb97mv_fast_gb300.scf import DeviceRKS
    mol = dimer('synthetic-svp')
    return mol, DeviceRKS(mol, levels=dict(xc=1, sgx=0, nlc=0),
                          coarse=dict(xc=0, sgx=0))


def test_fock_build_matches_oracle_on_a_fixed_density():
    import torch
    from oracle.scf import HostScf
    from pyscf_wb97mv_fast_gb300.grids import build_grids
    mol, rks = _dimer_case()
    grids = {k: build_grids(mol, level=lv) for k, lv in (('xc', 1), ('sgx', 0), ('nlc', 0))}
    host = HostScf(mol, grids)
    D = host.diag(host.H)
    E_ref, F_ref = host.fock(D)
    dg = rks._stage_grids(2)
    E, F, _, _ = rks.fock(torch.as_tensor(D, device=rks.device), dg, fp64=True)
    # the screens (k_tile_tol 1e-11, Hartree 1e-14) move single Fock
    # elements by up to ~1e-10 of max|F|; the energy by less
    scale = np.abs(F_ref).max()
    assert abs(float(E) - E_ref) < 1e-9
    assert np.abs(F.cpu().numpy() - F_ref).max() < 1e-9 * scale
    E32, F32, _, _ = rks.fock(torch.as_tensor(D, device=rks.device), dg, fp64=False)
    assert abs(float(E32) - E_ref) < 1e-5
    assert np.abs(F32.cpu().numpy() - F_ref).max() < 1e-6 * scale


def test_fp64_and_mixed_scf_reach_the_oracle_energy_water_dimer():
    mol, rks = _dimer_case()
    e_ref = _golden()['water_dimer_svp_xc1_sgx0_nlc0']['e_tot']
    r64 = rks.kernel(precision='fp64', reference_energy=e_ref)
    assert r64['converged']
    assert abs(r64['error_vs_reference']) < 1e-9, r64['error_vs_reference']
    rmx = rks.kernel(precision='mixed', reference_energy=e_ref)
    assert rmx['converged']
    assert abs(rmx['error_vs_reference']) < 1e-8, rmx['error_vs_reference']
    # the staged run went through S0, S1, S2 and the FP64 tail
    assert [s['stage'] for s in rmx['stages']][:2] == [0, 1]
    assert rmx['history'][-1]['fp64']


def test_incremental_builds_reach_the_same_energy():
    """Incremental builds from a fixed full-build base (the plain FP64
    form: FP64 increments of K; the staged form's tail: FP32 increments of
    K, J and rho on an FP64 base) converge to the energy of full builds, to
    well inside the 1e-8 Ha gate."""
    mol, rks = _dimer_case()
    e_ref = _golden()['water_dimer_svp_xc1_sgx0_nlc0']['e_tot']
    full = rks.kernel(precision='fp64', incremental=False)
    inc = rks.kernel(precision='fp64', incremental=True, profile=True)
    assert full['converged'] and inc['converged']
    assert abs(full['e_tot'] - inc['e_tot']) < 1e-9
    assert set(inc['profile']) >= {'k', 'j', 'xc'}
    mix_full = rks.kernel(precision='mixed', incremental=False)
    mix_inc = rks.kernel(precision='mixed', incremental=True)
    for r in (mix_full, mix_inc):
        assert r['converged'] and abs(r['e_tot'] - e_ref) < 2e-9, r['e_tot'] - e_ref


def test_mixed_scf_water8_svp_reaches_the_oracle_energy():
    """The molecule and grids: 8 seeded waters, synthetic def2-SVP
    (192 AOs), XC level 2, SGX level 1, VV10 level 1."""
    from pyscf_wb97mv_fast_gb300.basis import Molecule
    from pyscf_wb97mv_fast_gb300.scf import DeviceRKS
    from pyscf_wb97mv_fast_gb300.systems import water_cluster
    g = _golden().get('water8_svp_xc2_sgx1_nlc1')
    if g is None:
        pytest.skip('no oracle energy fixture for water8')
    mol = Molecule.build(water_cluster(8, box=7.0, seed=8), 'synthetic-svp')
    rks = DeviceRKS(mol, levels=dict(xc=2, sgx=1, nlc=1))
    r = rks.kernel(precision='mixed', reference_energy=g['e_tot'])
    assert r['converged']
    assert abs(r['error_vs_reference']) < 1e-8, r['error_vs_reference']


def test_fp64_and_mixed_scf_with_f_shells_reach_the_oracle_energy():
    """Ethane in the synthetic def2-TZVP structure (98 AOs, f shells on C):
    every (l_A, l_B) class up to (3, 3) in K, the one-electron integrals
    and the Hartree potential up to L = 6."""
    from pyscf_wb97mv_fast_gb300.basis import Molecule
    from pyscf_wb97mv_fast_gb300.scf import DeviceRKS
    from pyscf_wb97mv_fast_gb300.systems import alkane
    e_ref = _golden()['ethane_tzvp_xc1_sgx0_nlc0']['e_tot']
    mol = Molecule.build(alkane(2), 'synthetic-tzvp')
    rks = DeviceRKS(mol, levels=dict(xc=1, sgx=0, nlc=0), coarse=dict(xc=0, sgx=0))
    r64 = rks.kernel(precision='fp64', reference_energy=e_ref)
    assert r64['converged']
    assert abs(r64['error_vs_reference']) < 1e-9, r64['error_vs_reference']
    rmx = rks.kernel(precision='mixed', reference_energy=e_ref)
    assert rmx['converged']
    assert abs(rmx['error_vs_reference']) < 1e-8, rmx['error_vs_reference']


def test_reference_stage_table_switches_grids():
    """stage_levels (the reference's per-stage XC / SGX / NLC table): S0
    without VV10 on its own grids, S2 on the final ones; the mixed form
    still reaches the plain FP64 form's energy on the final grids."""
    from pyscf_wb97mv_fast_gb300.scf import DeviceRKS
    mol = dimer('synthetic-svp')
    table = dict(xc=(0, 1, 1), sgx=(0, 0, 1), nlc=(None, 0, 1))
    rks = DeviceRKS(mol, stage_levels=table)
    assert rks.levels == dict(xc=1, sgx=1, nlc=1)
    g0, g1, g2 = (rks._stage_grids(s) for s in (0, 1, 2))
    assert g0['nlc'] is None and g1['nlc'] is not None
    assert g1['sgx'] is g0['sgx'] and g2['sgx'] is not g1['sgx']
    r64 = rks.kernel(precision='fp64')
    rmx = rks.kernel(precision='mixed', reference_energy=r64['e_tot'])
    assert r64['converged'] and rmx['converged']
    assert [s['stage'] for s in rmx['stages']][:2] == [0, 1]
    assert abs(rmx['error_vs_reference']) < 1e-8, rmx['error_vs_reference']
