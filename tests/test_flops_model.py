"""The algorithmic flop model on hand counts (CPU)."""
import numpy as np

from pyscf_wb97mv_fast_gb300.flops_model import pair_flops_table, task_flops


def test_ss_hand_count():
    # f_prim = 11 + 14 + 0 + (1 + 3 + 1) + 2 = 32; + 2 (bra transform) + 4
    assert task_flops(0, 0, 1, 1, False) == 38
    assert task_flops(0, 0, 1, 1, True) == 36
    # K primitive pairs scale f_prim, npi scales the bra transform
    assert task_flops(0, 0, 5, 3, False) == 15 * 32 + 5 * 2 + 4


def test_ps_hand_count():
    # L = 1: 11 + 28 + 3 * (5 - 2) = 48; Hermite: x and y (2 + 6 + 1),
    # z (1 + 6 + 1) = 26; ket transform 2 * 3 * 1 * 1 = 6 -> f_prim 80;
    # bra 2 * 3 * 1 * 3 = 18; G contraction 4 * 3 * 1 = 12
    assert task_flops(1, 0, 1, 1, False) == 80 + 18 + 12


def test_pair_table_size_and_symmetry():
    from helpers import dimer
    mol = dimer()
    t = pair_flops_table(mol)
    nb = mol.nbas
    assert t.shape == (nb * (nb + 1) // 2,)
    assert np.all(t > 0)


def test_oracle_work_credit_matches_the_native_count():
    """The CPU baselines credit the work from the oracle's pair cut and the
    pure-Python model (so the reference arm loads no product library); it
    equals the native library's count of the same pairs."""
    import oracle
    from pyscf_wb97mv_fast_gb300.basis import Molecule
    from pyscf_wb97mv_fast_gb300.cosx import model_flops_per_point
    from pyscf_wb97mv_fast_gb300.systems import water_cluster, water_dimer
    mols = [Molecule.build(water_dimer(), 'synthetic-svp'),
            Molecule.build(water_dimer(), 'synthetic-tzvp'),
            Molecule.build(water_dimer(), 'synthetic-svp', gen_contract=True),
            Molecule.build(water_cluster(8, box=7.0, seed=8), 'synthetic-svp')]
    for m in mols:
        assert oracle.model_flops_per_point(m) == model_flops_per_point(m)
