#!/usr/bin/env python
"""COSX G-kernel benchmark (the workload of the reference's G microbench):

  27 seeded waters (O-H 0.9572 A, HOH 104.52 deg, oxygens uniform in a 10 A
  cube with O-O >= 2.7 A, random orientations), def2-SVP-structured basis
  (648 AOs), atom-centred grid (~3.8e5 points), D = 2 C C^T with C (648, 135)
  seeded N(0, 1) and orthonormalised, proj = identity, F = fl32(X D),
  screening k_tile_tol = 1e-11.

One step = the two K builds of one SCF cycle (full 1/r and erf(w r)/r,
w = 0.3) from one density: FP64 AO values -> F GEMM -> block stats, formed
once, then per omega the fused screen + G kernels -> K GEMM, all on the
device (wb_cosx_get_k_multi; --per-omega runs one wb_cosx_get_k per omega,
forming AO values and F twice).  The metric is COSX G TFLOP/s: the
algorithmic flop model of the kept (sub-block, shell pair) tasks
(pyscf_wb97mv_fast_gb300/flops_model.py) divided by the step time.

  value  : device-resident inputs, the K builds through the engine
  e2e    : host (pinned) coordinates, weights and density matrix copied in
           and both K matrices copied out every step, through
           GpuKBuilder/get_k_only_gpu-equivalent calls
  roofline: the G phase alone (wb_cosx_g_multi: block statistics, the
           fused screen + G class kernels of both omegas in one two-omega
           pass, the class-buffer sums), CUDA events on the launching
           stream, against the FP32 FMA peak measured in the same run
           (wb_fp32_fma_probe)
  cpu_baseline: the FP64 OpenMP oracle on a bounded sample of the points

--impl reference times the reference's CPU path for this workload on the
host cores.  PySCF (the reference's CPU implementation) is not installed,
so it is the C/OpenMP restatement of it (the oracle port), on a bounded
sample per step, same metric and unit.

Multi-GPU (torchrun, N > 1): replicas -- every rank runs the same workload
on its own GPU; value = sum of the per-rank work / max time over ranks.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

NWATER, BOX, SEED = 27, 10.0, 27
GRID_LEVEL = 2
NOCC = 135
OMEGAS = (0.0, 0.3)
TILE_TOL = 1e-11
METRIC = 'COSX G TFLOP/s (algorithmic flop model of kept tasks)'
UNIT = 'TFLOP/s'


def workload(small=False, grid_level=None, partition=None):
    from pyscf_wb97mv_fast_gb300.basis import Molecule
    from pyscf_wb97mv_fast_gb300.grids import build_grids
    from pyscf_wb97mv_fast_gb300.systems import water_cluster
    if small:
        mol = Molecule.build(water_cluster(8, box=7.0, seed=8), 'synthetic-svp')
        g = build_grids(mol, level=1 if grid_level is None else grid_level,
                        partition=partition)
        nocc = 40
    else:
        mol = Molecule.build(water_cluster(NWATER, box=BOX, seed=SEED),
                             'synthetic-svp')
        g = build_grids(mol, level=GRID_LEVEL if grid_level is None else grid_level,
                        partition=partition)
        nocc = NOCC
    rng = np.random.default_rng(SEED)
    c, _ = np.linalg.qr(rng.normal(size=(mol.nao, nocc)))
    dm = 2.0 * c @ c.T
    return mol, g, dm


class ClockSampler:
    """nvidia-smi clocks and throttle reasons during the timed region."""

    FIELDS = ('clocks.sm,clocks.max.sm,power.draw,'
              'clocks_event_reasons.hw_slowdown,'
              'clocks_event_reasons.hw_thermal_slowdown,'
              'clocks_event_reasons.sw_thermal_slowdown,'
              'clocks_event_reasons.sw_power_cap')

    def __init__(self, index=0):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ['nvidia-smi', '-i', str(self.index), '--query-gpu=' + self.FIELDS,
                 '--format=csv,noheader,nounits', '-lms', '200'],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, smax, reasons = [], None, set()
        names = ['hw_slowdown', 'hw_thermal_slowdown', 'sw_thermal_slowdown',
                 'sw_power_cap']
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(',')]
            if len(parts) < 7:
                continue
            try:
                sm.append(float(parts[0]))
                smax = float(parts[1])
            except ValueError:
                continue
            for nm, v in zip(names, parts[3:7]):
                if v.lower().startswith('active'):
                    reasons.add(nm)
        return {'sm_mhz': statistics.median(sm) if sm else None,
                'sm_max_mhz': smax, 'reasons': sorted(reasons),
                'samples': len(sm)}


def max_over_ranks(t, world, device):
    """The job's time: the slowest rank's (all-reduce MAX over the ranks of
    the default process group; the local time when world is 1)."""
    if world <= 1:
        return float(t)
    import torch
    import torch.distributed as dist
    tt = torch.tensor([float(t)], dtype=torch.float64, device=device)
    dist.all_reduce(tt, op=dist.ReduceOp.MAX)
    return float(tt.item())


def replica_throughput(work_per_rank, t_max, world):
    """Whole-job throughput of world replicas that each did
    work_per_rank in at most t_max seconds (weak scaling: the path does not
    shard, every rank runs the full workload on its own GPU)."""
    return world * float(work_per_rank) / float(t_max)


def measured_peaks():
    path = os.path.join(ROOT, 'MEASURED_PEAKS.json')
    if os.path.exists(path):
        with open(path) as fh:
            return json.load(fh)
    return None


FP32_PROBES = {}


def fp32_peak(torch):
    """FP32 FMA throughput of this GPU (TFLOP/s): best of 5 launches of the
    scalar-FMA probe and of the packed-FMA (fma.rn.f32x2) probe, the larger
    of the two (both kept in FP32_PROBES)."""
    from pyscf_wb97mv_fast_gb300 import _native
    lib = _native.lib()
    nsm = torch.cuda.get_device_properties(0).multi_processor_count
    out = torch.empty(nsm * 2048, dtype=torch.float32, device='cuda')
    flops = _native.ctypes.c_double()
    stream = _native.ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    for name, fn in (('ffma', lib.wb_fp32_fma_probe), ('ffma2', lib.wb_fp32x2_fma_probe)):
        best = 0.0
        for it in range(7):
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record()
            _native.check(fn(20000, _native.ptr(out), out.numel(), stream,
                             _native.ctypes.byref(flops)))
            e1.record()
            e1.synchronize()
            if it >= 2:
                best = max(best, flops.value / (e0.elapsed_time(e1) * 1e-3) / 1e12)
        FP32_PROBES[name] = best
    return max(FP32_PROBES.values())


def traffic_from_profile():
    path = os.path.join(ROOT, 'profiles', 'cosx_g_water27_traffic.json')
    if os.path.exists(path):
        with open(path) as fh:
            return json.load(fh)
    return None


def cpu_baseline(mol, g, dm, engine, budget_s=15.0):
    """FP64 oracle G on a bounded sample of the grid, both omegas.  Work
    credited as on the GPU: the model flops of the shell pairs kept by the
    reference's 1e-14 pair cut (the oracle computes those, all of them: no
    task screening)."""
    import oracle
    flops_per_pt, _ = oracle.model_flops_per_point(mol)
    cores = os.cpu_count() or 1
    rng = np.random.default_rng(1)
    X_idx = rng.choice(g.size, 64, replace=False)
    t0 = time.perf_counter()
    run_sample(oracle, mol, g, dm, X_idx)
    t_probe = time.perf_counter() - t0
    n = int(max(64, min(g.size, 64 * budget_s / max(t_probe, 1e-3))))
    idx = np.sort(rng.choice(g.size, n, replace=False))
    t0 = time.perf_counter()
    run_sample(oracle, mol, g, dm, idx)
    dt = time.perf_counter() - t0
    work = flops_per_pt * n * len(OMEGAS)
    return {'value': work / dt / 1e12, 'unit': UNIT, 'cores': cores,
            'kind': 'port',
            'sample': '%d of %d grid points, omega in %s, FP64 oracle, every '
                      'shell pair kept by the 1e-14 pair cut (no task '
                      'screening), OpenMP %d threads'
                      % (n, g.size, list(OMEGAS), cores),
            'seconds': dt}


class SlaterGgaTau:
    """Host stand-in for the functional of the semilocal flow timing
    (PySCF's libxc is not installed): Slater exchange plus a gradient and a
    kinetic-energy-density term, libxc convention."""

    def eval(self, rho):
        r = np.maximum(rho[0], 1e-12)
        sigma = (rho[1:4] ** 2).sum(axis=0)
        ex = np.exp(-r)
        cx = 0.7385587663820224
        e = -cx * r ** (4.0 / 3.0) + 0.05 * sigma * ex + 0.2 * rho[4] * r / (1.0 + r)
        vrho = (-4.0 / 3.0 * cx * r ** (1.0 / 3.0) - 0.05 * sigma * ex
                + 0.2 * rho[4] / (1.0 + r) ** 2)
        return e / r, vrho, 0.05 * ex, 0.2 * r / (1.0 + r)


def xc_flow_timing(mol, g, dm, eng, torch, calls=3):
    """Wall time of one semilocal XC flow (gpu_nr_rks, MGGA) on the bench
    molecule and grid, device synchronised; the host functional is the
    stand-in above."""
    import types
    from pyscf_wb97mv_fast_gb300.gpu.xc import XcContext, gpu_nr_rks

    class Ni:
        @staticmethod
        def _xc_type(xc_code):
            return 'MGGA'
    ctx = XcContext(mol, functional_factory=lambda xc, ni: SlaterGgaTau())
    ctx.engine = eng
    grids = types.SimpleNamespace(coords=g.coords, weights=g.weights)
    out = gpu_nr_rks(ctx, Ni(), mol, grids, 'mgga', dm)     # warm-up
    ts = []
    for _ in range(calls):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        out = gpu_nr_rks(ctx, Ni(), mol, grids, 'mgga', dm)
        torch.cuda.synchronize()
        ts.append(time.perf_counter() - t0)
    return {'ms_per_call': 1e3 * statistics.median(ts), 'calls': calls,
            'npts': int(g.size), 'nao': int(mol.nao), 'xctype': 'MGGA',
            'nelec': out[0],
            'functional': 'host stand-in (Slater exchange + gradient + tau '
                          'terms; PySCF libxc not installed)',
            'note': 'wall time per gpu_nr_rks call: AO values and gradients, '
                    '4 F-type GEMM splits, density pass, host functional, '
                    'Fock-side pass, 4 K-type GEMM splits'}


def vv10_timing(mol, dm, eng, torch, peak, calls=2):
    """The VV10 double sum (Vv10Kernel.kernel_sum, every pair kept) on the
    bench density's own VV10 terms over the level-1 grid: pairs/s and the
    27-operations-per-pair work (24 flops + 3 reciprocals) against the FP32
    peak measured in the same run."""
    from pyscf_wb97mv_fast_gb300.grids import build_grids
    from pyscf_wb97mv_fast_gb300.gpu.vv10 import THRESH, Vv10Kernel, vv10_pointwise
    g1 = build_grids(mol, level=1)
    c = eng.relative(g1.coords)
    n = int(g1.size)
    ao = eng.ao_eval_deriv1(c)[:, :, :n]
    D = torch.as_tensor(dm, device=eng.device)
    T = D @ ao[0]
    rho0 = (T * ao[0]).sum(dim=0)
    grad = 2.0 * torch.einsum('mp,dmp->dp', T, ao[1:4])
    del ao, T
    w = torch.as_tensor(g1.weights, device=eng.device)
    ind = rho0 >= THRESH
    q, W0, kappa = vv10_pointwise(rho0[ind], grad[:, ind], w[ind], (6.0, 0.01))[:3]
    xyz = c[ind].to(torch.float32)
    kern = Vv10Kernel(0.0)
    kern.kernel_sum(xyz, q, W0, kappa)
    ts = []
    for _ in range(calls):
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record()
        kern.kernel_sum(xyz, q, W0, kappa)
        e1.record()
        e1.synchronize()
        ts.append(e0.elapsed_time(e1) * 1e-3)
    t = min(ts)
    m = int(xyz.shape[0])
    pairs = float(m) * m
    tflops = 27.0 * pairs / t / 1e12
    out = {'points': m, 'grid': 'level 1 (%d points, rho >= %g kept)' % (n, THRESH),
           'ms_per_call': t * 1e3, 'pairs_per_s': pairs / t,
           'achieved_tflops': tflops, 'peak_tflops': peak,
           'frac': tflops / peak if peak else None,
           'work': '27 operations per pair (24 flops + 3 reciprocals), '
                   'every pair kept (tile_tol 0)',
           'parameters': 'b = 6.0, C = 0.01 (the wB97M-V VV10 set)'}
    # the distance-pruned sum (the reference's tile-pair bounds,
    # gpu/vv10.py:21-31): time, kept pairs and the change of the VV10
    # energy's pair term, E_F = 1/2 sum_i q_i F_i (F = -1.5 x the raw sum)
    F0 = kern.kernel_sum(xyz, q, W0, kappa)[0]
    e_full = 0.5 * float((q.to(torch.float64) * F0).sum())
    pruned = {}
    for tol in (1e-12, 1e-10, 1e-8):
        kp = Vv10Kernel(tol)
        kp.kernel_sum(xyz, q, W0, kappa)
        tp = []
        for _ in range(calls):
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record()
            Fp = kp.kernel_sum(xyz, q, W0, kappa)[0]
            e1.record()
            e1.synchronize()
            tp.append(e0.elapsed_time(e1) * 1e-3)
        kept, total = kp.last_pairs_kept
        e_p = 0.5 * float((q.to(torch.float64) * Fp).sum())
        pruned['%g' % tol] = {'ms_per_call': min(tp) * 1e3,
                              'pairs_kept_fraction': kept / total if total else None,
                              'dE_pair_term_Ha': e_p - e_full}
    out['distance_pruned'] = pruned
    return out


def fp64_form_timing(eng, coords_d, w_d, qd_d, K_mixed, t_mixed, dm, torch,
                     calls=2):
    """The plain FP64 form of the same step (wb_cosx_get_k_fp64: FP64 AO
    values, F kept in FP64, the same screen, FP64 G kernels, cuBLAS DGEMMs)
    on the same inputs: its time per step, its model-flop rate, the
    mixed-precision step's speed-up over it, and the mixed-precision K's
    deviation from it (max |dK| / max |K| and 1/4 tr(D dK) per omega)."""
    eng.get_k_fp64(coords_d, w_d, qd_d, OMEGAS, tile_tol=TILE_TOL)   # tables, warm-up
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(calls):
        K64 = eng.get_k_fp64(coords_d, w_d, qd_d, OMEGAS, tile_tol=TILE_TOL,
                             stats=False)
    e1.record()
    torch.cuda.synchronize()
    t = e0.elapsed_time(e1) / 1e3 / calls
    eng.get_k_fp64(coords_d, w_d, qd_d, OMEGAS, tile_tol=TILE_TOL)
    st = eng.last_stats
    dev = {}
    for i, w in enumerate(OMEGAS):
        a = ((K_mixed[i] + K_mixed[i].T) * 0.5).cpu().numpy()
        b = ((K64[i] + K64[i].T) * 0.5).cpu().numpy()
        dev['omega=%g' % w] = {
            'max_abs_dK_rel': float(np.abs(a - b).max() / np.abs(b).max()),
            'quarter_tr_D_dK': float(0.25 * np.einsum('ij,ji->', dm, a - b))}
    return {'ms_per_step': t * 1e3, 'model_flops_per_step': st['model_flops'],
            'tflops': st['model_flops'] / t / 1e12,
            'tasks_kept': st['pairs_kept'], 'tasks_total': st['pairs_total'],
            'mixed_speedup': t / t_mixed, 'mixed_vs_fp64': dev,
            'what': 'wb_cosx_get_k_fp64, both omegas, tile_tol %g, same inputs' % TILE_TOL}


def serving_requests(n_solves=16, cycles=3, seed=5):
    """Seeded SCF-shaped requests of uneven size: water clusters of 4-32
    waters (synthetic def2-SVP) and all-trans alkanes C6-C14 (synthetic
    def2-TZVP, f shells), level-0 grids, `cycles` exchange builds each with
    seeded densities (D = 2 C C^T, C orthonormal with the molecule's
    occupied count)."""
    from pyscf_wb97mv_fast_gb300.basis import Molecule
    from pyscf_wb97mv_fast_gb300.grids import build_grids
    from pyscf_wb97mv_fast_gb300.systems import alkane, water_cluster
    rng = np.random.default_rng(seed)
    out = []
    for i in range(n_solves):
        if rng.random() < 0.5:
            n = int(rng.integers(4, 33))
            mol = Molecule.build(water_cluster(n, box=max(5.0, 3.2 * n ** (1.0 / 3.0)),
                                               seed=100 + i), 'synthetic-svp')
            nocc, name = 5 * n, 'water%d/svp' % n
        else:
            n = int(rng.integers(6, 15))
            mol = Molecule.build(alkane(n), 'synthetic-tzvp')
            nocc, name = 4 * n + 1, 'C%dH%d/tzvp' % (n, 2 * n + 2)
        g = build_grids(mol, level=0)
        dms = []
        for c in range(cycles):
            r = np.random.default_rng(seed * 1000 + i * 10 + c)
            q, _ = np.linalg.qr(r.normal(size=(mol.nao, nocc)))
            dms.append(2.0 * q @ q.T)
        out.append((name, mol, g.coords, g.weights, dms))
    return out


def graph_timing(torch, sizes=(4, 8, 16, 32), reps=10):
    """Per-build time of a multi-omega K build (both omegas, level-0 grid,
    synthetic def2-SVP water clusters) launched directly vs replayed from
    its CUDA graph (CosxEngine.capture_k_multi), symmetrisation included."""
    from pyscf_wb97mv_fast_gb300.basis import Molecule
    from pyscf_wb97mv_fast_gb300.cosx import CosxEngine
    from pyscf_wb97mv_fast_gb300.grids import build_grids
    from pyscf_wb97mv_fast_gb300.systems import water_cluster
    out = {}
    for n in sizes:
        mol = Molecule.build(water_cluster(n, box=max(5.0, 3.2 * n ** (1.0 / 3.0)),
                                           seed=200 + n), 'synthetic-svp')
        g = build_grids(mol, level=0)
        eng = CosxEngine(mol)
        c = eng.relative(g.coords)
        w = torch.as_tensor(g.weights, device=eng.device)
        r = np.random.default_rng(n)
        q, _ = np.linalg.qr(r.normal(size=(mol.nao, 5 * n)))
        qd = torch.as_tensor(2.0 * q @ q.T, device=eng.device)
        K = torch.empty((len(OMEGAS), mol.nao, mol.nao), dtype=torch.float64,
                        device=eng.device)

        def direct():
            eng.get_k_multi(c, w, qd, OMEGAS, tile_tol=TILE_TOL, out=K, stats=False)
            return (K + K.transpose(1, 2)) * 0.5

        for _ in range(3):
            direct()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(reps):
            direct()
        torch.cuda.synchronize()
        t_direct = (time.perf_counter() - t0) / reps
        kg = eng.capture_k_multi(c, w, OMEGAS, tile_tol=TILE_TOL)
        for _ in range(3):
            kg.run(qd)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(reps):
            kg.run(qd)
        torch.cuda.synchronize()
        t_graph = (time.perf_counter() - t0) / reps
        same = bool(torch.equal(kg.run(qd), direct()))
        out['water%d' % n] = {'nao': mol.nao, 'points': int(g.size),
                              'direct_ms': t_direct * 1e3, 'graph_ms': t_graph * 1e3,
                              'bitwise_equal': same}
        del kg, eng
    return out


def grad_timing(torch, calls=2):
    """The COSX exchange nuclear gradient (wb_cosx_k_grad, FP64, grid
    response off) of the bench molecule and density on its level-0 grid,
    omega = 0, k_tile_tol as the K builds: ms per call after one warm-up
    call."""
    from pyscf_wb97mv_fast_gb300.cosx import CosxEngine
    from pyscf_wb97mv_fast_gb300.grids import build_grids
    mol, _, dm = workload()
    g0 = build_grids(mol, level=0)
    eng = CosxEngine(mol)
    c = eng.relative(g0.coords)
    w = torch.as_tensor(g0.weights, device=eng.device)
    grad = eng.k_grad(c, w, dm, 0.0, tile_tol=TILE_TOL)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(calls):
        grad = eng.k_grad(c, w, dm, 0.0, tile_tol=TILE_TOL)
    t = (time.perf_counter() - t0) / calls
    eng._ws = None
    eng.close()
    return {'ms_per_call': t * 1e3, 'points': int(g0.size), 'natm': mol.natm,
            'omega': 0.0, 'k_tile_tol': TILE_TOL,
            'max_abs_grad': float(np.abs(grad).max()),
            'what': 'AO values and gradients, F = X D, FP64 G, the AO-side '
                    'contraction, FP64 integral-derivative kernels'}


def batched_timing(torch, nmol=64, seed=4, iters=3):
    """Config-4 shape: nmol seeded water clusters of n in {4..32} waters
    (uniform), synthetic def2-SVP, level-0 grids, both omegas.  One SCF
    iteration's K builds of all molecules: one molecule per call
    (wb_cosx_get_k_multi, back to back on one stream) vs batched
    (wb_cosx_batch_run: one launch per class over the molecules of a wave;
    waves fill half of the free device memory with workspaces)."""
    from pyscf_wb97mv_fast_gb300.basis import Molecule
    from pyscf_wb97mv_fast_gb300.cosx import CosxBatch, CosxEngine, batch_workspace_bytes
    from pyscf_wb97mv_fast_gb300.grids import build_grids
    from pyscf_wb97mv_fast_gb300.systems import water_cluster
    rng = np.random.default_rng(seed)
    sizes = [int(x) for x in rng.integers(4, 33, size=nmol)]
    engines, grids, qds = [], [], []
    for i, n in enumerate(sizes):
        mol = Molecule.build(water_cluster(n, box=max(5.0, 3.2 * n ** (1.0 / 3.0)),
                                           seed=300 + i), 'synthetic-svp')
        g = build_grids(mol, level=0)
        eng = CosxEngine(mol)
        engines.append(eng)
        grids.append((eng.relative(g.coords), torch.as_tensor(g.weights, device=eng.device)))
        r = np.random.default_rng(seed * 1000 + i)
        q, _ = np.linalg.qr(r.normal(size=(mol.nao, 5 * n)))
        qds.append(torch.as_tensor(2.0 * q @ q.T, device=eng.device))
    wsb = [e.workspace_bytes(int(c.shape[0])) for e, (c, _) in zip(engines, grids)]
    wsb_batch, scratch = batch_workspace_bytes(engines, [int(c.shape[0]) for c, _ in grids])
    # one molecule per call, one shared workspace
    shared = torch.empty(max(wsb), dtype=torch.uint8, device=engines[0].device)
    outs = [torch.empty((len(OMEGAS), e.nao, e.nao), dtype=torch.float64,
                        device=e.device) for e in engines]
    for e in engines:
        e._ws = shared

    def per_molecule():
        for e, (c, w), q, o in zip(engines, grids, qds, outs):
            e.get_k_multi(c, w, q, OMEGAS, tile_tol=TILE_TOL, out=o, stats=False)

    def timed(fn):
        fn()
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(iters):
            fn()
        e1.record()
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / iters

    t_single = timed(per_molecule)
    ref = [o.clone() for o in outs]
    flops = 0.0
    for e, (c, w), q, o in zip(engines, grids, qds, outs):
        e.get_k_multi(c, w, q, OMEGAS, tile_tol=TILE_TOL, out=o, stats=True)
        flops += e.last_stats['model_flops']
    for e in engines:
        e._ws = None
    del shared
    torch.cuda.empty_cache()
    free, _ = torch.cuda.mem_get_info(engines[0].device)

    def plan(budget):
        waves, cur, used = [], [], scratch
        for i, b in enumerate(wsb_batch):
            if cur and used + b > budget:
                waves.append(cur)
                cur, used = [], scratch
            cur.append(i)
            used += b
        waves.append(cur)
        return waves

    # as few waves as the free HBM allows: 85 % of it first, fewer bytes per
    # wave if the workspaces do not fit after all
    for frac in (0.85, 0.6, 0.4):
        waves = plan(frac * free)
        try:
            batches = [CosxBatch([engines[i] for i in wv], [grids[i] for i in wv],
                                 OMEGAS, tile_tol=TILE_TOL) for wv in waves]
            break
        except torch.OutOfMemoryError:
            batches = None
            for e in engines:
                e._ws = None
            torch.cuda.empty_cache()
    if batches is None:
        raise RuntimeError('batched leg: the workspaces do not fit')
    bouts = [[outs[i] for i in wv] for wv in waves]

    def batched():
        for bt, wv, bo in zip(batches, waves, bouts):
            bt.run([qds[i] for i in wv], out=bo)

    t_batch = timed(batched)
    same = all(torch.equal(a, b) for a, b in zip(outs, ref))
    kernel_launches = 0
    for bt, wv, bo in zip(batches, waves, bouts):
        bt.run([qds[i] for i in wv], out=bo, stats=True)
        kernel_launches += bt.last_stats['kernel_launches']
    for bt in batches:
        bt.close()
    for e in engines:
        e._ws = None
    # the VV10 double sums of all molecules: one call per molecule vs one
    # batched launch (synthetic VV10 terms from an atom-centred model
    # density on each grid: q = w rho, W0 = sqrt(4 pi rho / 3), kappa = Kvv
    # rho^(1/6))
    from pyscf_wb97mv_fast_gb300.gpu.vv10 import Vv10Kernel
    vq, vw, vk = [], [], []
    kvv = 6.0 * 1.5 * np.pi * (9.0 * np.pi) ** (-1.0 / 6.0)
    for e, (c, w) in zip(engines, grids):
        r = torch.cdist(c, torch.as_tensor(e.mol.atom_coords() - e.origin,
                                           device=c.device))
        rho = torch.exp(-2.0 * r).sum(dim=1) + 1e-8
        vq.append(w * rho)
        vw.append(torch.sqrt(4.0 * np.pi / 3.0 * rho))
        vk.append(kvv * rho ** (1.0 / 6.0))
    vk1 = Vv10Kernel(0.0)
    vcs = [c.to(torch.float32) for c, _ in grids]

    def vv_single():
        return [vk1.kernel_sum(c, q, w0, k) for c, q, w0, k in zip(vcs, vq, vw, vk)]

    def vv_batch():
        return vk1.kernel_sum_batch(vcs, vq, vw, vk)

    t_vv1 = timed(vv_single)
    t_vvb = timed(vv_batch)
    single = vv_single()
    Fb, Ub, Wb = vv_batch()
    vv_same = all(torch.equal(a[0], b) for a, b in zip(single, Fb))
    vv_pairs = float(sum(int(c.shape[0]) ** 2 for c in vcs))
    for e in engines:
        e.close()
    return {'molecules': nmol, 'waters_per_cluster': sizes,
            'vv10_per_molecule_ms': t_vv1, 'vv10_batched_ms': t_vvb,
            'vv10_speedup': t_vv1 / t_vvb, 'vv10_pairs': vv_pairs,
            'vv10_bitwise_equal_to_per_molecule': bool(vv_same),
            'grid': 'level 0', 'points_total': int(sum(int(c.shape[0]) for c, _ in grids)),
            'waves': len(waves), 'workspace_gb': (sum(wsb_batch) + scratch) / 1e9,
            'per_molecule_ms_per_iteration': t_single,
            'batched_ms_per_iteration': t_batch, 'speedup': t_single / t_batch,
            'model_flops_per_iteration': flops,
            'tflops_batched': flops / (t_batch * 1e-3) / 1e12,
            'kernel_launches_batched': kernel_launches,
            'bitwise_equal_to_per_molecule': bool(same)}


def serving_timing(torch, rates=(4.0, 16.0), slots=4, seed=5):
    """Continuous batching of SCF-shaped requests (serving.ExchangeServer):
    the plain per-request form (one request at a time, back to back) and
    seeded Poisson arrivals at each rate with `slots` builds in flight;
    solves/s and p50/p99 time-to-result, and whether every served result is
    bitwise the result of the plain form."""
    from pyscf_wb97mv_fast_gb300.serving import (ExchangeServer, Solve,
                                                 poisson_arrivals, solve_summary)
    reqs = serving_requests(seed=seed)
    # warm-up: library, cuBLAS heuristics, pinned-memory pool
    srv = ExchangeServer(slots=1)
    Solve(srv, *reqs[0][1:4], reqs[0][4][:1]).run()
    srv.close()
    srv = ExchangeServer(slots=1)
    plain = [Solve(srv, m, c, w, d, tag=nm) for nm, m, c, w, d in reqs]
    for s in plain:
        s.run()
    srv.close()
    out = {'requests': [r[0] for r in reqs], 'cycles_per_solve': len(reqs[0][4]),
           'grid': 'level 0', 'omegas': list(OMEGAS), 'k_tile_tol': TILE_TOL,
           'plain': solve_summary(plain), 'served': {}}
    for rate in rates:
        srv = ExchangeServer(slots=slots)
        arr = poisson_arrivals(len(reqs), rate, seed)
        solves = [Solve(srv, m, c, w, d, tag=nm) for nm, m, c, w, d in reqs]
        t0 = time.perf_counter()
        for s, t in zip(solves, arr):
            dt = t0 + t - time.perf_counter()
            if dt > 0:
                time.sleep(dt)
            s.start()
        for s in solves:
            s.join()
        srv.close()
        same = all(all(np.array_equal(a, b) for a, b in zip(s.results, p.results))
                   for s, p in zip(solves, plain))
        summ = solve_summary(solves)
        summ.update({'rate_per_s': rate, 'slots': slots,
                     'max_concurrent_builds': srv.scheduler.max_running,
                     'bitwise_equal_to_plain': bool(same)})
        out['served']['rate=%g' % rate] = summ
    # the highest rate again with every session's builds captured in CUDA
    # graphs (first cycle captures, later cycles replay)
    rate = rates[-1]
    srv = ExchangeServer(slots=slots)
    arr = poisson_arrivals(len(reqs), rate, seed)
    solves = [Solve(srv, m, c, w, d, tag=nm, graphs=True) for nm, m, c, w, d in reqs]
    t0 = time.perf_counter()
    for s, t in zip(solves, arr):
        dt = t0 + t - time.perf_counter()
        if dt > 0:
            time.sleep(dt)
        s.start()
    for s in solves:
        s.join()
    srv.close()
    same = all(all(np.array_equal(a, b) for a, b in zip(s.results, p.results))
               for s, p in zip(solves, plain))
    summ = solve_summary(solves)
    summ.update({'rate_per_s': rate, 'slots': slots, 'cuda_graphs': True,
                 'max_concurrent_builds': srv.scheduler.max_running,
                 'bitwise_equal_to_plain': bool(same)})
    out['served']['rate=%g,graphs' % rate] = summ
    return out


def parity_vs_oracle(mol, g, dm, eng, torch, npts, seed=11):
    """The checker: max|dK|/max|K| and 1/4 tr(D dK) of the mixed-precision
    multi-omega K against the FP64 oracle on a seeded subset of the grid
    (same molecule, density, screen and kernels as the timed step).
    Untimed; the oracle runs on the host."""
    import oracle
    idx = np.sort(np.random.default_rng(seed).choice(g.size, npts, replace=False))
    coords, w = g.coords[idx], g.weights[idx]
    K = eng.get_k_multi(eng.relative(coords), torch.as_tensor(w, device=eng.device),
                        torch.as_tensor(dm, device=eng.device), OMEGAS,
                        tile_tol=TILE_TOL)
    K = (0.5 * (K + K.transpose(1, 2))).cpu().numpy()
    out = {'points': int(npts), 'of': int(g.size), 'seed': seed,
           'gates': 'max|dK| < 1e-6 max|K|; |dE| < 3e-7 (omega 0), 1e-7 (0.3) Ha'}
    for j, omega in enumerate(OMEGAS):
        ref = oracle.cosx_k(mol, coords, w, dm, omega)
        dk = K[j] - ref
        rel = float(np.abs(dk).max() / np.abs(ref).max())
        de = 0.25 * float(np.sum(dm * dk))
        out['omega=%g' % omega] = {
            'max_dK_over_max_K': rel, 'dE_quarter_tr_D_dK': de,
            'pass': bool(rel < 1e-6 and abs(de) < (3e-7 if omega == 0.0 else 1e-7))}
    return out


def alkane_timing(torch, peak, steps=3, n_carbon=20, level=2):
    """All-trans C20H42 in the def2-TZVP structure (f shells, every (3, x)
    class): one multi-omega K build per step on its level-2 grid, the G
    phase alone, per-class work, and parity on 1,000 points."""
    from pyscf_wb97mv_fast_gb300.basis import Molecule
    from pyscf_wb97mv_fast_gb300.cosx import CosxEngine, round32
    from pyscf_wb97mv_fast_gb300.grids import build_grids
    from pyscf_wb97mv_fast_gb300.systems import alkane
    mol = Molecule.build(alkane(n_carbon), 'synthetic-tzvp')
    g = build_grids(mol, level=level)
    rng = np.random.default_rng(20)
    c, _ = np.linalg.qr(rng.normal(size=(mol.nao, mol.nelectron // 2)))
    dm = 2.0 * c @ c.T
    eng = CosxEngine(mol)
    cd = eng.relative(g.coords)
    wd = torch.as_tensor(g.weights, device=eng.device)
    qd = torch.as_tensor(dm, device=eng.device)
    K = torch.empty((len(OMEGAS), mol.nao, mol.nao), dtype=torch.float64,
                    device=eng.device)

    def step():
        eng.get_k_multi(cd, wd, qd, OMEGAS, tile_tol=TILE_TOL, out=K, stats=False)
    step()
    eng.get_k_multi(cd, wd, qd, OMEGAS, tile_tol=TILE_TOL, out=K, stats=True,
                    profile=True)
    st = dict(eng.last_stats)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record()
    for _ in range(steps):
        step()
    e1.record()
    torch.cuda.synchronize()
    t_step = e0.elapsed_time(e1) / 1e3 / steps
    X = eng.ao_eval(cd)
    F = eng.ozaki_f(X, qd)
    del X
    Gt = torch.empty((len(OMEGAS), mol.nao, round32(g.size)), dtype=torch.float32,
                     device=eng.device)
    eng.g_multi(cd, wd, F, OMEGAS, TILE_TOL, out=Gt, stats=True)
    gst = dict(eng.last_stats)
    torch.cuda.synchronize()
    e0.record()
    for _ in range(steps):
        eng.g_multi(cd, wd, F, OMEGAS, TILE_TOL, out=Gt, stats=False)
    e1.record()
    torch.cuda.synchronize()
    t_g = e0.elapsed_time(e1) / 1e3 / steps
    del F, Gt
    g_tf = gst['model_flops'] / t_g / 1e12
    names = ['(%d,%d)' % (la, lb) for la in range(4) for lb in range(la + 1)]
    out = {
        'molecule': 'all-trans C%dH%d (C-C 1.53, C-H 1.09 A)' % (n_carbon, 2 * n_carbon + 2),
        'basis': 'synthetic def2-TZVP structure (f shells)', 'nao': mol.nao,
        'grid_points': int(g.size), 'grid_level': level, 'omegas': list(OMEGAS),
        'k_tile_tol': TILE_TOL,
        'ms_per_step': t_step * 1e3,
        'cosx_g_tflops_step': st['model_flops'] / t_step / 1e12,
        'g_phase_ms': t_g * 1e3, 'g_phase_tflops': g_tf,
        'g_roofline_frac_fp32': g_tf / peak if peak else None,
        'phases_ms': st.get('phase_ms'),
        'tasks_kept': st['pairs_kept'], 'tasks_total': st['pairs_total'],
        'classes': {names[c]: {'tasks_kept': gst['kept_class'][c],
                               'model_gflop': round(gst['flops_class'][c] / 1e9, 3),
                               'share': round(gst['flops_class'][c] /
                                              max(gst['model_flops'], 1), 4)}
                    for c in range(10) if gst['kept_class'][c]},
        'parity': parity_vs_oracle(mol, g, dm, eng, torch, 1000),
    }
    eng.close()
    return out


def reference_gpu_timing(g, eng, F, Gt, t_g, torch, vv10_points=209707):
    """The reference's own CUDA kernels on this GPU (oracle/ref_gpu: the
    extracted sgx_screen_mask, sgx_k_cls<LA,LB> and vv10_kernel_sum, built
    for sm_103a, launched with the reference's shapes) next to this
    library's, on the same grid, F and density; the G phases are
    cross-checked element by element."""
    from oracle.ref_gpu import runner
    why = runner.available()
    if why:
        return {'unavailable': why}
    ref = runner.RefGpu(device=eng.device.index or 0)
    n = g.size
    Fpm = F[:, :n].T.contiguous()                     # (npts, nao) point-major
    out = {'what': 'reference kernels extracted unmodified from gpu/sgx_k.py and '
                   'gpu/vv10.py, compiled with nvcc -arch=sm_103a; per 155,648-point '
                   'tile: sub-block stats + sgx_screen_mask (screen_ms), per-class CSR '
                   '(host round trips, csr_host_ms, not counted), sgx_k_cls launches '
                   '(class_kernels_ms)',
           'ours_g_phase_ms': t_g * 1e3}
    total = 0.0
    for j, omega in enumerate(OMEGAS):
        ref.g_phase(g.coords, g.weights, Fpm, omega, TILE_TOL)       # warm-up
        G, st = ref.g_phase(g.coords, g.weights, Fpm, omega, TILE_TOL)
        # compared as w o G, the quantity K = X^T (w o G) sees: the screens
        # (32-point sub-blocks there, 64-point blocks for the light
        # classes here) drop different tasks, each bounded by the
        # tolerance in w |A F|, not in |A F|
        wd = torch.as_tensor(g.weights, device=G.device)[:, None]
        mine = Gt[j][:, :n].T * wd
        G = G * wd
        scale = float(mine.abs().max())
        st['max_w_dG_vs_ours_over_max_wG'] = float((G - mine).abs().max()) / scale
        st['ms'] = st['screen_ms'] + st['class_kernels_ms']
        total += st['ms']
        out['omega=%g' % omega] = st
        del G
    out['ref_g_phase_ms'] = total
    out['speedup_g_phase'] = total / (t_g * 1e3)
    # VV10 double sum: both kernels on the same seeded inputs (every pair)
    rng = np.random.default_rng(31)
    xyz = torch.as_tensor(rng.uniform(-9.0, 9.0, (vv10_points, 3)), dtype=torch.float32,
                          device=eng.device)
    q, w0, kap = (torch.as_tensor(rng.uniform(lo, hi, vv10_points), dtype=torch.float32,
                                  device=eng.device)
                  for lo, hi in ((1e-6, 1e-2), (0.3, 3.0), (0.4, 2.0)))
    from pyscf_wb97mv_fast_gb300.gpu.vv10 import Vv10Kernel
    mine_k = Vv10Kernel(0.0)

    def tmin(fn, reps=3):
        fn()
        ts = []
        for _ in range(reps):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            fn()
            e1.record()
            torch.cuda.synchronize()
            ts.append(e0.elapsed_time(e1))
        return min(ts)
    t_ref = tmin(lambda: ref.vv10(xyz, q, w0, kap))
    t_mine = tmin(lambda: mine_k.kernel_sum(xyz, q, w0, kap))
    Fr, Ur, Wr = ref.vv10(xyz, q, w0, kap)
    Fm, Um, Wm = mine_k.kernel_sum(xyz, q, w0, kap)
    out['vv10'] = {'points': vv10_points, 'inputs': 'seeded uniform (every pair kept)',
                   'ref_ms': t_ref, 'ours_ms': t_mine, 'speedup': t_ref / t_mine,
                   'max_rel_diff_F': float(((-1.5 * Fr - Fm).abs() / Fm.abs()).max()),
                   'max_rel_diff_U': float(((Ur - Um).abs() / Um.abs()).max())}
    return out


def scf_timing(torch):
    """Eight seeded waters (synthetic def2-SVP, XC level 2, SGX
    level 1, VV10 level 1): the device SCF in its mixed-precision staged
    form and its plain FP64 form, each from the core guess to convergence;
    energies against the oracle's host SCF (tests/golden/scf_energies.json,
    oracle/scf.py); wall time to reach 1e-8 Ha of it."""
    from pyscf_wb97mv_fast_gb300.basis import Molecule
    from pyscf_wb97mv_fast_gb300.scf import DeviceRKS
    from pyscf_wb97mv_fast_gb300.systems import water_cluster
    path = os.path.join(ROOT, 'tests', 'golden', 'scf_energies.json')
    with open(path) as fh:
        golden = json.load(fh)
    ref = golden.get('water8_svp_xc2_sgx1_nlc1', {}).get('e_tot')
    mol = Molecule.build(water_cluster(8, box=7.0, seed=8), 'synthetic-svp')
    rks = DeviceRKS(mol, levels=dict(xc=2, sgx=1, nlc=1))
    # warm-up: grids, AO values and first launches (not timed)
    rks.kernel(precision='mixed', max_cycle=2)
    rks.kernel(precision='fp64', max_cycle=2)
    out = {'molecule': '8 seeded waters in a 7 A cube (seed 8), synthetic def2-SVP',
           'nao': mol.nao, 'levels': rks.levels, 'coarse': rks.coarse,
           'functional': rks.functional.name, 'oracle_energy': ref,
           'oracle': 'oracle/scf.py (host FP64, unscreened) via '
                     'tests/golden/scf_energies.json'}
    for form in ('mixed', 'fp64'):
        prof = rks.kernel(precision=form, profile=True)['profile']   # untimed
        r = rks.kernel(precision=form, reference_energy=ref)
        t_hit = None
        if ref is not None:
            for h in r['history']:
                if abs(h['e'] - ref) < 1e-8 and (form == 'fp64' or h['fp64']):
                    t_hit = h['t']
                    break
        out[form] = {'e_tot': r['e_tot'], 'error_vs_oracle': r.get('error_vs_reference'),
                     'converged': r['converged'], 'cycles': r['cycles'],
                     'wall_s': r['wall'], 'wall_to_1e-8_s': t_hit,
                     'cycles_fp64': sum(1 for h in r['history'] if h['fp64']),
                     'incremental_fp64_exchange': r['incremental'],
                     'profile_s': {k: round(v, 4) for k, v in prof.items()},
                     'stages': [{k: v for k, v in s.items()} for s in r['stages']]}
    m, f = out['mixed'], out['fp64']
    out['fp64_over_mixed_wall'] = f['wall_s'] / m['wall_s']
    if m['wall_to_1e-8_s'] and f['wall_to_1e-8_s']:
        out['fp64_over_mixed_to_1e-8'] = f['wall_to_1e-8_s'] / m['wall_to_1e-8_s']
    rks.eng.close()
    return out


def _scf_record(r, ref):
    """The per-form fields of an SCF leg: energy, error against ref, walls
    (whole run, and to the first FP64 cycle within 1e-8 Ha of ref)."""
    t_hit = None
    if ref is not None:
        for h in r['history']:
            if abs(h['e'] - ref) < 1e-8 and h['fp64']:
                t_hit = h['t']
                break
    tail = [h for h in r['history'] if h['fp64']][-30:]
    return {'e_tot': r['e_tot'], 'error_vs_reference': r.get('error_vs_reference'),
            'converged': r['converged'], 'cycles': r['cycles'], 'wall_s': r['wall'],
            'wall_to_1e-8_s': t_hit,
            'cycles_fp64': sum(1 for h in r['history'] if h['fp64']),
            'stages': [dict(s) for s in r['stages']],
            'fp64_cycles': [{'cycle': h['cycle'], 'err': h.get('err'), 'dE': h['dE'],
                             'gnorm': h['gnorm'], 't': round(h['t'], 3)} for h in tail]}


def scf_c20_timing(torch, n_carbon=20):
    """The staged mixed-precision SCF of all-trans C20H42 in the
    synthetic def2-TZVP structure (f shells) on the reference's per-stage
    grid table (XC 1/3/3, SGX 1/1/2, NLC off/1/3), against the plain FP64
    form on the final grids.  The host oracle SCF needs about 45 min for
    192 AOs, so the FP64 form's converged energy -- the form pinned to the
    oracle's SCF to 2e-10 Ha on eight waters in SVP and on an f-shell molecule in the
    GPU tests -- is the FP64 reference energy here.  Each form runs once
    from the core guess (per-part profile on); grids and AO values are
    built by an untimed warm-up."""
    from pyscf_wb97mv_fast_gb300.basis import Molecule
    from pyscf_wb97mv_fast_gb300.scf import DeviceRKS, REFERENCE_STAGE_LEVELS
    from pyscf_wb97mv_fast_gb300.systems import alkane
    mol = Molecule.build(alkane(n_carbon), 'synthetic-tzvp')
    rks = DeviceRKS(mol, stage_levels=REFERENCE_STAGE_LEVELS)
    t0 = time.perf_counter()
    for st in (0, 1, 2):
        grids = rks._stage_grids(st)
    setup = time.perf_counter() - t0
    rks.kernel(precision='mixed', max_cycle=1)
    rks.kernel(precision='fp64', max_cycle=1)
    r64 = rks.kernel(precision='fp64', profile=True)
    ref = r64['e_tot']
    rmx = rks.kernel(precision='mixed', profile=True, reference_energy=ref)
    r64['error_vs_reference'] = 0.0
    for h in r64['history']:
        h['err'] = h['e'] - ref
    out = {'molecule': 'all-trans C%dH%d (C-C 1.53, C-H 1.09 A)' % (n_carbon, 2 * n_carbon + 2),
           'basis': 'synthetic def2-TZVP structure (f shells)', 'nao': mol.nao,
           'stage_levels': {k: list(v) for k, v in REFERENCE_STAGE_LEVELS.items()},
           'grid_points': {'%s_level%d' % (k, lv): int(rks.grid(k, lv).n)
                           for k, v in REFERENCE_STAGE_LEVELS.items() for lv in set(v)
                           if lv is not None},
           'grid_setup_s': setup, 'functional': rks.functional.name,
           'reference_energy': ref,
           'reference': 'the plain FP64 device form on the final grids (pinned to the '
                        'host oracle SCF on eight waters/SVP and on ethane/TZVP)'}
    out['mixed'] = _scf_record(rmx, ref)
    out['mixed']['profile_s'] = {k: round(v, 3) for k, v in rmx['profile'].items()}
    out['fp64'] = _scf_record(r64, ref)
    out['fp64']['profile_s'] = {k: round(v, 3) for k, v in r64['profile'].items()}
    out['fp64_over_mixed_wall'] = r64['wall'] / rmx['wall']
    m, f = out['mixed'], out['fp64']
    if m['wall_to_1e-8_s'] and f['wall_to_1e-8_s']:
        out['fp64_over_mixed_to_1e-8'] = f['wall_to_1e-8_s'] / m['wall_to_1e-8_s']
    rks.eng.close()
    return out


def scf_batched_timing(torch, nmol=64, seed=4, wave=16, max_waters=32):
    """nmol seeded water clusters of n in {4..32} waters
    (uniform), synthetic def2-SVP, XC level 1 / SGX level 0 / VV10 level 0
    (S0 on XC 0 / SGX 0), every molecule a full SCF.  The plain FP64 form of
    each molecule (its own SCF, one after another) gives its FP64 reference
    energy; the mixed staged form runs one molecule at a time and batched
    (BatchedRKS: the FP32 exchange builds of all molecules in one batched
    build per SGX level, their VV10 double sums in one launch).  A batch
    keeps every molecule's grids and AO values resident (about 3.5 GB for
    a 20-water cluster), so the molecules run in waves of `wave`; walls
    are summed over the waves.  Grids and AO values are built by an
    untimed warm-up."""
    from pyscf_wb97mv_fast_gb300.basis import Molecule
    from pyscf_wb97mv_fast_gb300.scf import BatchedRKS
    from pyscf_wb97mv_fast_gb300.systems import water_cluster
    rng = np.random.default_rng(seed)
    sizes = [int(x) for x in rng.integers(4, max_waters + 1, size=nmol)]
    levels, coarse = dict(xc=1, sgx=0, nlc=0), dict(xc=0, sgx=0)
    t64 = tseq = tb = 0.0
    errs, conv, equal, cyc_m, cyc_f, nb, nao_tot = [], True, True, [], [], 0, 0

    def timed(fn):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        out = fn()
        torch.cuda.synchronize()
        return out, time.perf_counter() - t0

    for w0 in range(0, nmol, wave):
        mols = [Molecule.build(water_cluster(n, box=max(5.0, 3.2 * n ** (1.0 / 3.0)),
                                             seed=300 + i), 'synthetic-svp')
                for i, n in list(enumerate(sizes))[w0:w0 + wave]]
        b = BatchedRKS(mols, levels=levels, coarse=coarse)
        b.kernel(precision='mixed', max_cycle=1)       # warm-up: grids, batches
        for r in b.rks:
            r.kernel(precision='fp64', max_cycle=1)
        r64, t = timed(lambda: [r.kernel(precision='fp64') for r in b.rks])
        t64 += t
        print('scf_batched: wave %d: FP64 SCFs %.1f s' % (w0 // wave, t), file=sys.stderr,
              flush=True)
        refs = [r['e_tot'] for r in r64]
        rseq, t = timed(lambda: [r.kernel(precision='mixed', reference_energy=e)
                                 for r, e in zip(b.rks, refs)])
        tseq += t
        rb = b.kernel(precision='mixed', reference_energies=refs)
        tb += rb[0]['batch_wall']
        print('scf_batched: wave %d: mixed one by one %.1f s, batched %.1f s'
              % (w0 // wave, t, rb[0]['batch_wall']), file=sys.stderr, flush=True)
        errs += [r['error_vs_reference'] for r in rb]
        conv = conv and all(r['converged'] for r in rb + r64)
        equal = equal and all(a['e_tot'] == c['e_tot'] for a, c in zip(rb, rseq))
        cyc_m += [r['cycles'] for r in rb]
        cyc_f += [r['cycles'] for r in r64]
        nb += rb[0]['batched_exchange_builds']
        nao_tot += int(sum(r.mol.nao for r in b.rks))
        b.close()
        del b, r64, rseq, rb
        torch.cuda.empty_cache()
    return {'molecules': nmol, 'waters_per_cluster': sizes, 'wave': wave,
            'max_waters': max_waters,
            'levels': levels, 'coarse': coarse, 'nao_total': nao_tot,
            'reference': "each molecule's plain FP64 device SCF on the final grids",
            'fp64_sequential_wall_s': t64,
            'mixed_sequential_wall_s': tseq,
            'mixed_batched_wall_s': tb,
            'fp64_over_mixed_batched': t64 / tb,
            'batched_over_sequential_speedup': tseq / tb,
            'all_converged': conv,
            'max_abs_error_vs_fp64_Ha': max(abs(e) for e in errs),
            'all_within_1e-8': all(abs(e) < 1e-8 for e in errs),
            'batched_equals_sequential': equal,
            'cycles_mixed': cyc_m, 'cycles_fp64': cyc_f,
            'batched_exchange_builds': nb}


def serving_scf_timing(torch, n_req=12, rates=(2.0, 8.0), slots=4, seed=7):
    """Config-5 shape with whole SCF solves as requests (ScfServer): a
    seeded mix of water clusters (4-12 waters, synthetic def2-SVP) and
    n-alkanes (C6-C10, synthetic def2-TZVP), XC level 1 / SGX 0 / VV10 0.
    The plain per-request form solves them one after another (one slot);
    the served form takes Poisson arrivals into `slots` overlapping solves.
    Reports solves/s and p50 / p99 time to the converged energy, and
    whether every served energy is bitwise its plain solve's."""
    from pyscf_wb97mv_fast_gb300.basis import Molecule
    from pyscf_wb97mv_fast_gb300.serving import ScfServer, poisson_arrivals, replay
    from pyscf_wb97mv_fast_gb300.systems import alkane, water_cluster
    rng = np.random.default_rng(seed)
    mols, names = [], []
    for i in range(n_req):
        if rng.random() < 0.5:
            n = int(rng.integers(4, 13))
            mols.append(Molecule.build(water_cluster(n, box=max(5.0, 3.2 * n ** (1 / 3)),
                                                     seed=500 + i), 'synthetic-svp'))
            names.append('water%d/svp' % n)
        else:
            c = int(rng.integers(6, 11))
            mols.append(Molecule.build(alkane(c), 'synthetic-tzvp'))
            names.append('C%dH%d/tzvp' % (c, 2 * c + 2))
    levels, coarse = dict(xc=1, sgx=0, nlc=0), dict(xc=0, sgx=0)
    warm = ScfServer(slots=1, levels=levels, coarse=coarse)
    warm.submit(mols[0]).result()
    warm.close()
    plain = ScfServer(slots=1, levels=levels, coarse=coarse)
    pf = [plain.submit(m) for m in mols]
    pr = [f.result() for f in pf]
    plain.close()
    out = {'requests': names, 'levels': levels, 'coarse': coarse,
           'plain': plain.summary(), 'served': {}}
    for rate in rates:
        srv = ScfServer(slots=slots, levels=levels, coarse=coarse)
        arr = poisson_arrivals(n_req, rate, seed)
        futs = replay([lambda m=m: srv.submit(m) for m in mols], arr)
        res = [f.result() for f in futs]
        srv.close()
        sm = srv.summary()
        sm['rate_per_s'] = rate
        sm['bitwise_equal_to_plain'] = all(a['e_tot'] == b['e_tot']
                                           for a, b in zip(pr, res))
        sm['all_converged'] = all(r['converged'] for r in res)
        out['served']['rate=%g' % rate] = sm
    return out


def run_sample(oracle, mol, g, dm, idx):
    coords = g.coords[idx]
    X = oracle.ao_eval(mol, coords)
    F = X @ dm
    for w in OMEGAS:
        oracle.cosx_g(mol, coords, F, w)


def run_reference(args):
    """--impl reference: the CPU restatement of the reference's path."""
    rank = int(os.environ.get('RANK', '0'))
    if rank != 0:
        return
    import oracle
    mol, g, dm = workload(args.small, partition=oracle.becke_partition)
    # model flops per point of the pairs kept by the reference's 1e-14 pair
    # cut (the CPU path does no task screening); the oracle and the
    # pure-Python flop model count them, so this arm loads no product code
    flops_per_pt, _ = oracle.model_flops_per_point(mol)
    cores = os.cpu_count() or 1
    rng = np.random.default_rng(2)
    npts = args.ref_points
    times = []
    for step in range(args.warmup + args.steps):
        idx = np.sort(rng.choice(g.size, npts, replace=False))
        t0 = time.perf_counter()
        run_sample(oracle, mol, g, dm, idx)
        if step >= args.warmup:
            times.append(time.perf_counter() - t0)
    tstep = sum(times) / len(times)
    value = flops_per_pt * npts * len(OMEGAS) / tstep / 1e12
    line = {
        'impl': 'reference', 'metric': METRIC, 'value': value, 'unit': UNIT,
        'n_gpus': args.gpus, 'steps': args.steps, 'warmup': args.warmup,
        'ms_per_step': tstep * 1e3, 'higher_is_better': True,
        'scaling': 'weak', 'vs_baseline': None, 'dtype': 'f64',
        'data': 'synthetic',
        'config': config_dict(mol, g, args),
        'cpu_baseline': {'value': value, 'unit': UNIT, 'cores': cores,
                         'kind': 'port',
                         'sample': '%d of %d grid points per step, both omegas, '
                                   'every shell pair kept by the 1e-14 pair cut, '
                                   'FP64 C/OpenMP restatement of the reference '
                                   'path (PySCF absent)' % (npts, g.size)},
        'e2e': {'value': value, 'unit': UNIT, 'h2d_bytes_per_step': 0,
                'd2h_bytes_per_step': 0},
    }
    print(json.dumps(line))


def config_dict(mol, g, args):
    return {'workload': 'cosx_g_water%d_svp' % (8 if args.small else NWATER),
            'molecule': '%d seeded waters in a %.0f A cube (seed %d)'
                        % (8 if args.small else NWATER, 7.0 if args.small else BOX,
                           8 if args.small else SEED),
            'basis': 'synthetic def2-SVP structure', 'nao': mol.nao,
            'grid_points': int(g.size), 'omegas': list(OMEGAS),
            'k_tile_tol': TILE_TOL, 'proj': 'identity',
            'omega_builds': 'per-omega' if getattr(args, 'per_omega', False)
                            else 'multi-omega (shared AO values and F)',
            'l2': 'inputs larger than L2 (X alone is %.1f GB)'
                  % (8.0 * mol.nao * g.size / 1e9),
            'gemm': args.gemm, 'f_engine': args.f_engine, 'parallelism': 'replicas'}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument('--gpus', type=int, default=1)
    ap.add_argument('--steps', type=int, default=5)
    ap.add_argument('--warmup', type=int, default=3)
    ap.add_argument('--impl', default='ours', choices=['ours', 'reference'])
    ap.add_argument('--gemm', default='ozaki', choices=['ozaki', 'native', 'emulated'])
    ap.add_argument('--f-engine', default='library', choices=['library', 'tc'],
                    help="the Ozaki F product: this library's tcgen05 kernel or "
                         "cuBLAS level GEMMs (bitwise the same F)")
    ap.add_argument('--small', action='store_true',
                    help='8 waters / grid level 1 (profiling captures)')
    ap.add_argument('--grid-level', type=int, default=None,
                    help='grid level (profiling captures of a smaller grid)')
    ap.add_argument('--no-cpu-baseline', action='store_true')
    ap.add_argument('--per-omega', action='store_true',
                    help='one get_k call per omega instead of one multi-omega '
                         'call (AO values and F formed twice)')
    ap.add_argument('--ref-points', type=int, default=400)
    ap.add_argument('--no-xc', action='store_true',
                    help='skip the semilocal XC flow timing')
    ap.add_argument('--no-fp64', action='store_true',
                    help='skip the plain FP64 form timing')
    ap.add_argument('--no-serving', action='store_true',
                    help='skip the continuous-batching serving leg')
    ap.add_argument('--no-grad', action='store_true',
                    help='skip the exchange-gradient timing')
    ap.add_argument('--no-autotune', action='store_true',
                    help='keep the compiled-in per-class kernel variants')
    ap.add_argument('--no-batched', action='store_true',
                    help='skip the batched (many molecules per launch) leg')
    ap.add_argument('--no-alkane', action='store_true',
                    help='skip the C20H42 / def2-TZVP (f shells) leg')
    ap.add_argument('--no-scf', action='store_true',
                    help='skip the device SCF leg (8 waters / SVP, mixed vs FP64)')
    ap.add_argument('--scf-batched', type=int, default=0, metavar='N',
                    help='add the batched-SCF leg over N water clusters in waves '
                         'of 16 (each molecule also runs its plain FP64 '
                         'SCF: about 20 s a molecule)')
    ap.add_argument('--scf-batched-max-waters', type=int, default=32,
                    help='largest cluster of the batched-SCF leg')
    ap.add_argument('--serving-scf', action='store_true',
                    help='add the served-SCF leg (whole SCF solves as requests)')
    ap.add_argument('--scf-c20', action='store_true',
                    help='add the C20H42 / def2-TZVP staged SCF leg ('
                         'minutes: its plain FP64 run is the reference energy)')
    ap.add_argument('--no-reference-gpu', action='store_true',
                    help="skip the reference's own kernels on this GPU")
    ap.add_argument('--no-parity', action='store_true',
                    help='skip the oracle check of K on a grid subset')
    ap.add_argument('--batched-molecules', type=int, default=64,
                    help='water clusters in the batched leg (profiling: fewer)')
    args = ap.parse_args()
    if args.impl == 'reference':
        return run_reference(args)

    import torch
    import torch.distributed as dist
    world = int(os.environ.get('WORLD_SIZE', '1'))
    rank = int(os.environ.get('RANK', '0'))
    local = int(os.environ.get('LOCAL_RANK', '0'))
    torch.cuda.set_device(local)
    if world > 1:
        dist.init_process_group('nccl')

    from pyscf_wb97mv_fast_gb300 import build as _build
    _build.build()
    from pyscf_wb97mv_fast_gb300.cosx import CosxEngine, round32, set_f_engine
    set_f_engine(args.f_engine)

    mol, g, dm = workload(args.small, args.grid_level)
    eng = CosxEngine(mol, device=local)
    dev = eng.device
    coords_d = eng.relative(g.coords)
    w_d = torch.as_tensor(g.weights, device=dev)
    qd_d = torch.as_tensor(dm, device=dev)
    # per-class kernel variants tuned on this grid and density (untimed set-up)
    tuned = None
    if not args.no_autotune:
        from pyscf_wb97mv_fast_gb300.autotune import autotune_classes
        tuned = autotune_classes(eng, coords_d, w_d, qd_d, OMEGAS, tile_tol=TILE_TOL)
        torch.cuda.empty_cache()
    K = torch.empty((len(OMEGAS), mol.nao, mol.nao), dtype=torch.float64,
                    device=dev)

    def build_k(c, wt, q, stats=False, profile=False):
        # both omegas of one density: one multi-omega call (AO values, F and
        # block statistics shared), or one call per omega with --per-omega
        if args.per_omega:
            sts = []
            for i, w in enumerate(OMEGAS):
                eng.get_k(c, wt, q, w, tile_tol=TILE_TOL, gemm=args.gemm,
                          out=K[i], stats=stats, profile=profile)
                sts.append(eng.last_stats)
            return sts
        eng.get_k_multi(c, wt, q, OMEGAS, tile_tol=TILE_TOL, gemm=args.gemm,
                        out=K, stats=stats, profile=profile)
        return [eng.last_stats]

    def step():
        build_k(coords_d, w_d, qd_d)

    # warm the library (cuBLAS heuristics, first launches), then one counted
    # and profiled build: kept tasks, model flops, launches, phases
    step()
    torch.cuda.synchronize()
    flops_step, launches_step, kept, total = 0.0, 0, 0, 0
    phases = {}
    kept_cls = [0] * 10
    flops_cls = [0.0] * 10
    for st in build_k(coords_d, w_d, qd_d, stats=True, profile=True):
        flops_step += st['model_flops']
        launches_step += st['kernel_launches']
        kept += st['pairs_kept']
        total += st['pairs_total']
        for c in range(10):
            kept_cls[c] += st['kept_class'][c]
            flops_cls[c] += st['flops_class'][c]
        for k, v in st['phase_ms'].items():
            phases[k] = phases.get(k, 0.0) + v

    def timed(fn, steps, warmup):
        for _ in range(warmup):
            fn()
        if world > 1:
            dist.barrier()
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(steps):
            fn()
        e1.record()
        torch.cuda.synchronize()
        if world > 1:
            dist.barrier()
        return e0.elapsed_time(e1) / 1e3 / steps

    with ClockSampler(local) as clocks:
        t_step = timed(step, args.steps, args.warmup)
    t_step = max_over_ranks(t_step, world, dev)
    value = replica_throughput(flops_step, t_step, world) / 1e12

    # -- e2e: pinned host inputs in, K out, every step ----------------------------
    coords_rel_h = (g.coords - eng.origin).astype(np.float64)
    c_h = torch.from_numpy(np.ascontiguousarray(coords_rel_h)).pin_memory()
    w_h = torch.from_numpy(np.ascontiguousarray(g.weights)).pin_memory()
    d_h = torch.from_numpy(np.ascontiguousarray(dm)).pin_memory()
    k_h = [torch.empty((mol.nao, mol.nao), dtype=torch.float64).pin_memory()
           for _ in OMEGAS]
    c_d2 = torch.empty_like(coords_d)
    w_d2 = torch.empty_like(w_d)
    q_d2 = torch.empty_like(qd_d)

    def e2e_step():
        c_d2.copy_(c_h, non_blocking=True)
        w_d2.copy_(w_h, non_blocking=True)
        q_d2.copy_(d_h, non_blocking=True)
        build_k(c_d2, w_d2, q_d2)
        for i in range(len(OMEGAS)):
            Ks = (K[i] + K[i].T) * 0.5
            k_h[i].copy_(Ks, non_blocking=True)

    t_e2e = timed(e2e_step, args.steps, 1)
    t_e2e = max_over_ranks(t_e2e, world, dev)
    h2d = c_h.numel() * 8 + w_h.numel() * 8 + d_h.numel() * 8
    d2h = sum(k.numel() * 8 for k in k_h)

    # -- roofline of the G phase (wb_cosx_g_multi on the same F) -----------------
    n = g.size
    ld = round32(n)
    X = eng.ao_eval(coords_d)
    F = eng.ozaki_f(X, qd_d)                    # fl32(X QD), AO-major
    Gt = torch.empty((len(OMEGAS), mol.nao, ld), dtype=torch.float32,
                     device=dev)
    # both omegas in one call, as in the step: block statistics once, the
    # omega pair in one pass of the two-omega class kernels
    eng.g_multi(coords_d, w_d, F, OMEGAS, TILE_TOL, out=Gt, stats=True)
    g_flops = eng.last_stats['model_flops']
    g_launches = eng.last_stats['kernel_launches']

    def g_step():
        eng.g_multi(coords_d, w_d, F, OMEGAS, TILE_TOL, out=Gt, stats=False)
    t_g = timed(g_step, max(2, args.steps), 1)
    del X
    refgpu = None if args.no_reference_gpu else reference_gpu_timing(g, eng, F, Gt, t_g,
                                                                     torch)
    peak = fp32_peak(torch)
    achieved = g_flops / t_g / 1e12
    prof = traffic_from_profile()
    roofline = {'bound': 'fp32', 'achieved': achieved, 'peak': peak,
                'unit': 'TFLOP/s', 'frac': achieved / peak if peak else None,
                'traffic': prof.get('bytes_per_g_phase') if prof else None,
                'traffic_source': prof.get('source') if prof else None,
                'peak_source': 'measured in this run: the larger of '
                               'wb_fp32_fma_probe (scalar FMAs) and '
                               'wb_fp32x2_fma_probe (packed f32x2 FMAs), all SMs',
                'fp32_probes_tflops': dict(FP32_PROBES),
                'kernel': 'block statistics + fused screen + G class kernels '
                          '+ class-buffer sums of both omegas in one call '
                          '(wb_cosx_g_multi, %d launches)' % g_launches,
                'ms': t_g * 1e3}
    mp = measured_peaks()
    if mp:
        roofline['measured_peaks_file'] = {'hbm_gbs': mp.get('hbm_gbs'),
                                           'bf16_tflops': mp.get('bf16_tflops')}

    xc_flow = None if args.no_xc else xc_flow_timing(mol, g, dm, eng, torch)
    vv10 = None if args.no_xc else vv10_timing(mol, dm, eng, torch, peak)
    build_k(coords_d, w_d, qd_d)
    fp64_form = None if args.no_fp64 else fp64_form_timing(
        eng, coords_d, w_d, qd_d, K, t_step, dm, torch)
    serving = None if (args.no_serving or world > 1) else serving_timing(torch)
    graphs = None if (args.no_serving or world > 1) else graph_timing(torch)
    eng._ws = None
    torch.cuda.empty_cache()
    batched = None if (args.no_batched or world > 1) else batched_timing(
        torch, nmol=args.batched_molecules)
    k_grad = None if (args.no_grad or world > 1) else grad_timing(torch)
    alk = None if (args.no_alkane or world > 1) else alkane_timing(torch, peak)
    torch.cuda.empty_cache()
    scf = None if (args.no_scf or world > 1) else scf_timing(torch)
    scf_c20 = scf_c20_timing(torch) if (args.scf_c20 and world == 1) else None
    scf_batched = (scf_batched_timing(torch, args.scf_batched,
                                      max_waters=args.scf_batched_max_waters)
                   if (args.scf_batched > 0 and world == 1) else None)
    serving_scf = serving_scf_timing(torch) if (args.serving_scf and world == 1) else None
    torch.cuda.empty_cache()
    parity = None if args.no_parity else parity_vs_oracle(mol, g, dm, eng, torch, 3000)

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        cpu = cpu_baseline(mol, g, dm, eng)

    if rank == 0:
        line = {
            'metric': METRIC, 'value': value, 'unit': UNIT, 'n_gpus': world,
            'steps': args.steps, 'warmup': args.warmup,
            'ms_per_step': t_step * 1e3, 'higher_is_better': True,
            'scaling': 'weak', 'vs_baseline': None, 'dtype': 'f32',
            'data': 'synthetic (seeded generators; no PySCF grids or basis)',
            'config': config_dict(mol, g, args),
            'e2e': {'value': replica_throughput(flops_step, t_e2e, world) / 1e12,
                    'unit': UNIT,
                    'ms_per_step': t_e2e * 1e3, 'h2d_bytes_per_step': h2d,
                    'd2h_bytes_per_step': d2h},
            'roofline': roofline,
            'cpu_baseline': cpu,
            'xc_flow': xc_flow,
            'vv10': vv10,
            'fp64_form': fp64_form,
            'serving': serving,
            'cuda_graphs': graphs,
            'batched': batched,
            'autotune': tuned,
            'k_grad': k_grad,
            'alkane_c20_tzvp': alk,
            'scf': scf,
            'scf_c20h42_tzvp': scf_c20,
            'scf_batched': scf_batched,
            'serving_scf': serving_scf,
            'reference_gpu': refgpu,
            'parity_vs_fp64_oracle': parity,
            'clocks': clocks.summary(),
            'gpu_launches': launches_step * args.steps,
            'tasks_kept': kept, 'tasks_total': total,
            'model_flops_per_step': flops_step,
            'phases_ms_per_step': phases,
            'classes': {'(%d,%d)' % (la, lb): {
                'tasks_kept': kept_cls[la * (la + 1) // 2 + lb],
                'model_gflop': round(flops_cls[la * (la + 1) // 2 + lb] / 1e9, 3)}
                for la in range(4) for lb in range(la + 1)
                if kept_cls[la * (la + 1) // 2 + lb]},
        }
        print(json.dumps(line))
    if world > 1:
        dist.destroy_process_group()


if __name__ == '__main__':
    main()
