"""Writes tests/golden/scf_energies.json: converged energies of the oracle's
host SCF (oracle/scf.py: FP64, unscreened) on this project's seeded
molecules and grids, the reference energies of the device SCF tests and
the bench's SCF leg.

Run from the repository root (each case is merged into the file):
    python tests/golden/make_scf_golden.py [case ...]
Cases: water_dimer_svp_xc1_sgx0_nlc0, water8_svp_xc2_sgx1_nlc1,
ethane_tzvp_xc1_sgx0_nlc0 (f shells).
"""
import json
import os
import sys
import time

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from pyscf_wb97mv_fast_gb300.basis import Molecule  # noqa: E402
from pyscf_wb97mv_fast_gb300.grids import build_grids  # noqa: E402
from pyscf_wb97mv_fast_gb300.systems import alkane, water_cluster, water_dimer  # noqa: E402

CASES = {
    'water_dimer_svp_xc1_sgx0_nlc0': (lambda: water_dimer(), 'synthetic-svp', 1, 0, 0),
    'water8_svp_xc2_sgx1_nlc1': (lambda: water_cluster(8, box=7.0, seed=8),
                                 'synthetic-svp', 2, 1, 1),
    'ethane_tzvp_xc1_sgx0_nlc0': (lambda: alkane(2), 'synthetic-tzvp', 1, 0, 0),
}


def run(name):
    from oracle.scf import HostScf
    atoms, basis, xc, sgx, nlc = CASES[name]
    mol = Molecule.build(atoms(), basis)
    grids = {'xc': build_grids(mol, level=xc), 'sgx': build_grids(mol, level=sgx),
             'nlc': build_grids(mol, level=nlc)}
    t0 = time.perf_counter()
    r = HostScf(mol, grids).kernel(verbose=True)
    return {'e_tot': r['e_tot'], 'converged': r['converged'], 'cycles': r['cycles'],
            'nao': mol.nao, 'grid_points': {k: int(g.size) for k, g in grids.items()},
            'functional': 'rsh-lda-vv10 (0.15 K + 0.85 K(0.3), 0.85 SR-LDA x, VWN5, '
                          'VV10 b=6 C=0.01)',
            'oracle_seconds': round(time.perf_counter() - t0, 1)}


def main():
    path = os.path.join(HERE, 'scf_energies.json')
    data = {}
    if os.path.exists(path):
        with open(path) as fh:
            data = json.load(fh)
    for name in (sys.argv[1:] or list(CASES)):
        data[name] = run(name)
        with open(path, 'w') as fh:
            json.dump(data, fh, indent=1, sort_keys=True)
        print(name, data[name]['e_tot'])


if __name__ == '__main__':
    main()
