"""The multi-GPU path of the bench is replicas only (the COSX K build has
no exchange step between GPUs): every rank runs the whole workload, the
job's time is the slowest rank's, the throughput is world x the per-rank
work over it.  Checked with two gloo ranks on the CPU (127.0.0.1)."""
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    s = socket.socket()
    s.bind(('127.0.0.1', 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank(rank, world, port, out):
    import torch
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    import bench
    os.environ.update(MASTER_ADDR='127.0.0.1', MASTER_PORT=str(port))
    dist.init_process_group('gloo', rank=rank, world_size=world)
    try:
        t = [0.25, 0.75][rank]                      # the second rank is slower
        tmax = bench.max_over_ranks(t, world, torch.device('cpu'))
        out.put((rank, tmax, bench.replica_throughput(3.0e12, tmax, world)))
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_take_the_slowest_time():
    import torch.multiprocessing as mp
    pytest.importorskip('torch.distributed')
    ctx = mp.get_context('spawn')
    out = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, out)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    res = sorted(out.get(timeout=10) for _ in range(2))
    for rank, tmax, thr in res:
        assert tmax == 0.75
        assert thr == pytest.approx(2 * 3.0e12 / 0.75)


def test_single_rank_is_the_local_time():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.max_over_ranks(0.5, 1, None) == 0.5
    assert bench.replica_throughput(1.0e12, 0.5, 1) == 2.0e12
