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


def test_clock_summary_reads_nvidia_smi_samples():
    """The clocks key of the bench line: median SM clock under load, the
    maximum, and only throttle reasons that were Active (nvidia-smi csv,
    noheader, nounits; unreadable lines are skipped)."""
    import bench
    c = bench.ClockSampler()
    c.lines = ['2070, 2070, 650.1, Not Active, Not Active, Not Active, Not Active',
               '1980, 2070, 1390.5, Not Active, Not Active, Not Active, Active',
               '[N/A], 2070, 10.0, Not Active, Not Active, Not Active, Not Active',
               'garbage',
               '2055, 2070, 1200.0, Not Active, Not Active, Not Active, Not Active']
    s = c.summary()
    assert s == {'sm_mhz': 2055.0, 'sm_max_mhz': 2070.0,
                 'reasons': ['sw_power_cap'], 'samples': 3}
    c.lines = ['1200, 2070, 900.0, Active, Not Active, Active, Not Active']
    assert c.summary()['reasons'] == ['hw_slowdown', 'sw_thermal_slowdown']
    assert bench.ClockSampler().summary()['sm_mhz'] is None
