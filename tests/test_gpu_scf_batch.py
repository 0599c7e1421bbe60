"""BatchedRKS: the SCFs of several molecules in lockstep, their FP32
exchange builds batched per SGX grid level and their VV10 double sums in
one launch.  The batched builds are bitwise the per-molecule ones, so each
molecule's run is the one DeviceRKS makes alone: the same cycles and the
same energies, bitwise, through the stage switches and the FP64 tail."""
import pytest

from helpers import dimer, waters

pytestmark = pytest.mark.gpu

LEVELS = dict(xc=1, sgx=0, nlc=0)
COARSE = dict(xc=0, sgx=0)


def _mols():
    from pyscf_wb97mv_fast_gb300.basis import Molecule
    from pyscf_wb97mv_fast_gb300.systems import alkane
    return [dimer('synthetic-svp'), waters(3, box=6.0, seed=5),
            Molecule.build(alkane(2), 'synthetic-tzvp')]


@pytest.mark.parametrize('precision', ['mixed', 'fp64'])
def test_batched_scf_is_each_molecules_own_scf(precision):
    from pyscf_wb97mv_fast_gb300.scf import BatchedRKS, DeviceRKS
    mols = _mols()
    alone = [DeviceRKS(m, levels=LEVELS, coarse=COARSE).kernel(precision=precision)
             for m in mols]
    b = BatchedRKS(mols, levels=LEVELS, coarse=COARSE)
    try:
        res = b.kernel(precision=precision)
    finally:
        b.close()
    for a, r in zip(alone, res):
        assert r['converged'] and a['converged']
        assert r['cycles'] == a['cycles']
        assert r['e_tot'] == a['e_tot'], (r['e_tot'], a['e_tot'])
        assert [h['e'] for h in r['history']] == [h['e'] for h in a['history']]
    if precision == 'mixed':
        # the FP32 builds went through the batch
        assert res[0]['batched_exchange_builds'] > 0


def test_batched_scf_reaches_the_oracle_energy_of_each_molecule():
    """The water dimer and ethane/TZVP of the SCF fixtures, in one batch:
    each within 1e-8 Ha of its oracle energy."""
    import json
    import os
    from pyscf_wb97mv_fast_gb300.basis import Molecule
    from pyscf_wb97mv_fast_gb300.scf import BatchedRKS
    from pyscf_wb97mv_fast_gb300.systems import alkane
    here = os.path.dirname(os.path.abspath(__file__))
    with open(os.path.join(here, 'golden', 'scf_energies.json')) as fh:
        gold = json.load(fh)
    mols = [dimer('synthetic-svp'), Molecule.build(alkane(2), 'synthetic-tzvp')]
    refs = [gold['water_dimer_svp_xc1_sgx0_nlc0']['e_tot'],
            gold['ethane_tzvp_xc1_sgx0_nlc0']['e_tot']]
    with BatchedRKS(mols, levels=LEVELS, coarse=COARSE) as b:
        res = b.kernel(precision='mixed', reference_energies=refs)
        engines = [e for kb in b._kb.values() for e in kb.engines]
    assert engines and all(e._h is None for e in engines)
    for r in res:
        assert r['converged']
        assert abs(r['error_vs_reference']) < 1e-8, r['error_vs_reference']


def test_scf_server_solves_alone_and_in_the_mix_equal():
    """ScfServer: whole SCF solves as requests, three slots overlapping on
    the device; each molecule's energy is bitwise its solve alone."""
    from pyscf_wb97mv_fast_gb300.scf import DeviceRKS
    from pyscf_wb97mv_fast_gb300.serving import ScfServer
    mols = _mols()
    alone = [DeviceRKS(m, levels=LEVELS, coarse=COARSE).kernel()['e_tot'] for m in mols]
    srv = ScfServer(slots=3, levels=LEVELS, coarse=COARSE)
    try:
        futs = [srv.submit(m) for m in mols]
        res = [f.result(timeout=600) for f in futs]
    finally:
        srv.close()
    for a, r in zip(alone, res):
        assert r['converged']
        assert r['e_tot'] == a
    s = srv.summary()
    assert s['requests'] == 3 and s['max_concurrent'] >= 2
