"""Continuous batching on the GPU (serving.ExchangeServer): every request
returns bitwise the same K alone, in a mix of concurrent requests, and
through a direct engine call; the builds of different requests overlap."""
import numpy as np
import pytest

from helpers import density, dimer, grid_subset, waters

pytestmark = pytest.mark.gpu


def _cases():
    from pyscf_wb97mv_fast_gb300.basis import Molecule
    from pyscf_wb97mv_fast_gb300.systems import alkane
    mols = [waters(4, 5.0, 1), waters(6, 6.0, 2),
            Molecule.build(alkane(6), 'synthetic-tzvp'),
            dimer('synthetic-svp', True)]
    out = []
    for i, mol in enumerate(mols):
        coords, weights = grid_subset(mol, 0, 6000 - 1000 * i, 10 + i)
        dms = [density(mol.nao, 6, 20 + 3 * i + c) for c in range(2)]
        out.append((mol, coords, weights, dms))
    return out


def test_served_results_equal_alone_mix_and_direct():
    import torch
    from pyscf_wb97mv_fast_gb300.cosx import CosxEngine
    from pyscf_wb97mv_fast_gb300.serving import ExchangeServer, Solve
    cases = _cases()
    # alone: one request at a time
    srv1 = ExchangeServer(slots=1)
    alone = [Solve(srv1, m, c, w, d).run() for m, c, w, d in cases]
    srv1.close()
    assert srv1.scheduler.max_running == 1
    # mix: all solves at once, four builds in flight
    srv4 = ExchangeServer(slots=4)
    solves = [Solve(srv4, m, c, w, d).start() for m, c, w, d in cases]
    mixed = [s.join(120) for s in solves]
    srv4.close()
    assert srv4.scheduler.max_running >= 2
    for a, b in zip(alone, mixed):
        for ka, kb in zip(a, b):
            assert ka.shape == kb.shape
            assert np.array_equal(ka, kb)
    # direct engine call, same inputs
    mol, coords, weights, dms = cases[2]
    eng = CosxEngine(mol)
    K = eng.get_k_multi(eng.relative(coords),
                        torch.as_tensor(weights, device=eng.device),
                        torch.as_tensor(dms[1], device=eng.device), (0.0, 0.3),
                        tile_tol=1e-11)
    K = ((K + K.transpose(1, 2)) * 0.5).cpu().numpy()
    assert np.array_equal(K, alone[2][1])
    summ = srv4.summary()
    assert summ['requests'] == 8 and summ['p99_s'] >= summ['p50_s'] > 0


def test_budget_rejects_what_can_never_fit():
    from pyscf_wb97mv_fast_gb300.serving import ExchangeServer, Rejected
    mol, coords, weights, dms = _cases()[0]
    srv = ExchangeServer(slots=2)
    s = srv.open_session(mol, coords[:64], weights[:64])
    srv.scheduler.budget = s.resident + s.footprint - 1
    with pytest.raises(Rejected):
        s.submit(dms[0])
    srv.scheduler.budget = s.resident + s.footprint
    K = s.submit(dms[0]).result(60)
    assert K.shape == (2, mol.nao, mol.nao)
    s.close()
    srv.close()
    assert srv.scheduler.resident == 0


def test_captured_build_replays_match_direct_builds():
    """A K build captured in a CUDA graph replays bitwise the direct build,
    for each new density."""
    import torch
    from pyscf_wb97mv_fast_gb300.cosx import CosxEngine
    mol, coords, weights, dms = _cases()[1]
    eng = CosxEngine(mol)
    c = eng.relative(coords)
    w = torch.as_tensor(weights, device=eng.device)
    kg = eng.capture_k_multi(c, w, (0.0, 0.3), tile_tol=1e-11)
    for dm in (dms[0], dms[1], dms[0]):
        Kg = kg.run(dm).cpu().numpy()
        Kd = eng.get_k_multi(c, w, torch.as_tensor(dm, device=eng.device),
                             (0.0, 0.3), tile_tol=1e-11)
        Kd = ((Kd + Kd.transpose(1, 2)) * 0.5).cpu().numpy()
        assert np.array_equal(Kg, Kd)


def test_served_with_graphs_equal_plain():
    from pyscf_wb97mv_fast_gb300.serving import ExchangeServer, Solve
    cases = _cases()
    srv1 = ExchangeServer(slots=1)
    alone = [Solve(srv1, m, c, w, d + d[:1]).run() for m, c, w, d in cases]
    srv1.close()
    srv = ExchangeServer(slots=3)
    solves = [Solve(srv, m, c, w, d + d[:1], graphs=True).start()
              for m, c, w, d in cases]
    got = [s.join(120) for s in solves]
    srv.close()
    for a, b in zip(alone, got):
        for ka, kb in zip(a, b):
            assert np.array_equal(ka, kb)
