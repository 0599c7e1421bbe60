"""The per-class kernel-variant knobs and the autotuner on the GPU: every
variant gives the same K to FP32 rounding, the tuner leaves a variant set
per class and never ends slower than it started."""
import numpy as np
import pytest

from helpers import density, grid_subset, waters

pytestmark = pytest.mark.gpu


def test_variants_agree_and_autotuner_runs():
    import torch
    from pyscf_wb97mv_fast_gb300.autotune import (autotune_classes, get_variant,
                                                  set_variant, variant_name)
    from pyscf_wb97mv_fast_gb300.cosx import CosxEngine
    mol = waters(5, 6.0, 11)
    coords, weights = grid_subset(mol, 1, 20000, 12)
    dm = density(mol.nao, 20, 13)
    eng = CosxEngine(mol)
    c = eng.relative(coords)
    w = torch.as_tensor(weights, device=eng.device)
    qd = torch.as_tensor(dm, device=eng.device)
    K0 = eng.get_k_multi(c, w, qd, (0.0, 0.3), tile_tol=1e-11).cpu().numpy()
    scale = np.abs(K0).max()
    # every variant of every class (where the molecule can run it)
    for cls in range(6):
        if not eng.class_pairs[cls]:
            continue
        keep = get_variant(eng, cls)
        for v in ((1, 1), (1, 0), (0, 1), (0, 0)):
            if set_variant(eng, cls, *v):
                assert get_variant(eng, cls) == v
                K = eng.get_k_multi(c, w, qd, (0.0, 0.3), tile_tol=1e-11).cpu().numpy()
                assert np.max(np.abs(K - K0)) < 1e-6 * scale, (cls, v)
        assert set_variant(eng, cls, *keep)
    rep = autotune_classes(eng, c, w, qd, (0.0, 0.3), tile_tol=1e-11, reps=2)
    assert rep['g_ms_tuned'] <= rep['g_ms_default']
    names = {variant_name(v) for v in ((1, 1), (0, 1), (0, 0))}
    assert rep['classes'] and all(r['chosen'] in names
                                  for r in rep['classes'].values())
    K = eng.get_k_multi(c, w, qd, (0.0, 0.3), tile_tol=1e-11).cpu().numpy()
    assert np.max(np.abs(K - K0)) < 1e-6 * scale
    with pytest.raises(Exception):
        set_variant(eng, 11, 0, 0)
