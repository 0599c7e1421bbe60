"""Continuous batching of COSX exchange builds, and of whole SCF solves
(ScfServer), on one GPU.

The reference runs one SCF at a time.  Batch throughput is an explicit
non-goal there (docs/design.en.md:44), and its K builder serves one
molecule per call (gpu/sgx_k.py:663-751).  This module serves many
molecules at once.

* A *session* is one molecule whose state stays on the device between
  requests: the engine's packed shell pairs (the C-ABI handle) and the
  grid coordinates and weights.  This is the state an SCF keeps across
  cycles.
* A *request* is one exchange build of a session: a new density in, K for
  every omega of the session out (wb_cosx_get_k_multi).  This is the K
  work of one SCF cycle.

Requests that arrive while others run on the GPU are admitted as soon as a
slot and enough device memory are free.  Admission scans the queue in
arrival order and takes the first request that fits (first fit), so a
large request at the head does not stall small ones behind it.  A session
runs one request at a time, in submission order.  Each slot is a host
thread with its own CUDA stream, so the builds of different slots overlap
on the device.

Memory.  A running request holds its build's workspace
(wb_cosx_workspace_bytes), its density and its K buffers.  An open session
holds its pair tables and grid.  Admission keeps the sum of running
footprints plus the resident session bytes under the budget (default 60 %
of the free device memory, the reference's mem_fraction,
gpu/install.py:209).  A request whose session could never fit is rejected
at submit time.  A session is admitted only when one of its own requests
fits on top of it, so open sessions can never hold the whole budget while
their requests wait.

Determinism.  Every kernel of a build has a fixed summation order that
does not depend on launch shape, block order or what else runs on the
device.  So a request returns bitwise the same K alone and in a mix.

The scheduling core (Scheduler) is plain Python with no GPU.  The GPU
executor (ExchangeServer) plugs CosxEngine calls into it.
"""
import collections
import threading
import time

import numpy as np


class Rejected(ValueError):
    """A request that can never be admitted (its footprint exceeds the
    budget) or a server that is closed."""


class Cancelled(Exception):
    """A request cancelled before it started (Future.cancel)."""


class Expired(TimeoutError):
    """A request whose deadline passed before it started."""


class Future:
    """Result handle of one request."""

    def __init__(self, tag=None, sched=None):
        self.tag = tag
        self._sched = sched
        self._ev = threading.Event()
        self._value = None
        self._error = None
        self.t_submit = time.perf_counter()
        self.t_start = None
        self.t_done = None

    def _finish(self, value=None, error=None):
        self._value, self._error = value, error
        self.t_done = time.perf_counter()
        self._ev.set()

    def done(self):
        return self._ev.is_set()

    def cancel(self):
        """Drop the request if it has not started: True, and result()
        raises Cancelled.  False once it runs or is finished (a started
        build is never interrupted on the device)."""
        return self._sched is not None and self._sched._cancel(self)

    def result(self, timeout=None):
        if not self._ev.wait(timeout):
            raise TimeoutError('request not finished')
        if self._error is not None:
            raise self._error
        return self._value

    @property
    def latency(self):
        return None if self.t_done is None else self.t_done - self.t_submit

    @property
    def queued(self):
        return None if self.t_start is None else self.t_start - self.t_submit


class Scheduler:
    """Slots, a memory budget and a queue; GPU-free.

    run_fn(job, slot) executes one admitted job on worker `slot` (0 ..
    slots - 1) and returns its value.  Jobs carry .footprint (bytes while
    running) and .key (jobs with the same key run one at a time, in
    submission order).
    """

    def __init__(self, run_fn, slots=4, budget=None):
        if slots < 1:
            raise ValueError('slots must be >= 1')
        self.run_fn = run_fn
        self.slots = int(slots)
        self.budget = None if budget is None else int(budget)
        self.resident = 0                # bytes held outside running jobs
        self._queue = collections.deque()
        self._busy_keys = set()
        self._used = 0
        self._running = 0
        self._closed = False
        self._cv = threading.Condition()
        self.max_running = 0             # high-water marks (tests, reports)
        self.max_used = 0
        self._workers = [threading.Thread(target=self._worker, args=(i,),
                                          daemon=True, name='cosx-slot-%d' % i)
                         for i in range(self.slots)]
        for t in self._workers:
            t.start()

    # -- resident bytes (sessions) ------------------------------------------
    def reserve(self, nbytes, wait=False, timeout=None, headroom=0):
        """Hold nbytes outside running jobs (an open session).  headroom:
        bytes that must fit on top of it at admission -- the footprint of
        the session's own requests -- so that the most recently admitted
        session can always run once the others' jobs end, and sessions
        waiting on each other cannot starve every request.  wait: block
        until running jobs and other sessions leave room (a size above the
        whole budget is rejected at once); otherwise reject if it does not
        fit now."""
        need = int(nbytes) + int(headroom)
        with self._cv:
            if self.budget is not None:
                if need > self.budget or not wait:
                    if self.resident + need > self.budget:
                        raise Rejected('resident state of %d bytes (+ %d headroom) '
                                       'exceeds the budget (%d of %d bytes held)'
                                       % (nbytes, headroom, self.resident,
                                          self.budget))
                elif not self._cv.wait_for(
                        lambda: self._used + self.resident + need <= self.budget,
                        timeout):
                    raise Rejected('no room for %d resident bytes within %s s'
                                   % (nbytes, timeout))
            self.resident += int(nbytes)

    def release(self, nbytes):
        with self._cv:
            self.resident -= int(nbytes)
            self._cv.notify_all()

    # -- jobs ------------------------------------------------------------------
    def submit(self, job, tag=None, deadline=None):
        """Queue job; returns its Future.  deadline: seconds from now by
        which the job must have started, else it is dropped and result()
        raises Expired."""
        fut = Future(tag, self)
        t_end = None if deadline is None else fut.t_submit + float(deadline)
        with self._cv:
            if self._closed:
                raise Rejected('scheduler is closed')
            if self.budget is not None and job.footprint + self.resident > self.budget:
                raise Rejected('request footprint %d bytes (+ %d resident) exceeds '
                               'the budget of %d bytes' % (job.footprint,
                                                           self.resident, self.budget))
            self._queue.append((job, fut, t_end))
            self._cv.notify_all()
        return fut

    def _cancel(self, fut):
        with self._cv:
            for i, item in enumerate(self._queue):
                if item[1] is fut:
                    del self._queue[i]
                    fut._finish(error=Cancelled('request cancelled before it started'))
                    self._cv.notify_all()
                    return True
        return False

    def _expire(self, now):
        """Finish the queued jobs whose deadline has passed; returns the
        seconds to the next deadline (None: no deadline queued)."""
        keep, nxt = collections.deque(), None
        for item in self._queue:
            t_end = item[2]
            if t_end is not None and now >= t_end:
                item[1]._finish(error=Expired('request not started within its '
                                              'deadline'))
                continue
            if t_end is not None:
                nxt = t_end - now if nxt is None else min(nxt, t_end - now)
            keep.append(item)
        if len(keep) != len(self._queue):
            self._queue = keep
            self._cv.notify_all()
        return nxt

    def _fits(self, job):
        if job.key in self._busy_keys:
            return False
        if self.budget is None:
            return True
        return self._used + job.footprint + self.resident <= self.budget

    def _take(self):
        # first fit in arrival order; a key's jobs keep their order (an
        # earlier job of a busy or waiting key blocks its later ones)
        blocked = set()
        for i, (job, fut, _) in enumerate(self._queue):
            if job.key in blocked:
                continue
            if self._fits(job):
                del self._queue[i]
                return job, fut
            blocked.add(job.key)
        return None

    def _worker(self, slot):
        while True:
            with self._cv:
                item = None
                while not self._closed or self._queue:
                    wake = self._expire(time.perf_counter())
                    item = self._take()
                    if item is not None:
                        break
                    if self._closed and not self._queue:
                        break
                    self._cv.wait(wake)
                if item is None:
                    return
                job, fut = item
                self._busy_keys.add(job.key)
                self._used += job.footprint
                self._running += 1
                self.max_running = max(self.max_running, self._running)
                self.max_used = max(self.max_used, self._used + self.resident)
                fut.t_start = time.perf_counter()
            value, error = None, None
            try:
                value = self.run_fn(job, slot)
            except BaseException as e:           # noqa: BLE001 -- handed to the caller
                error = e
            with self._cv:
                self._busy_keys.discard(job.key)
                self._used -= job.footprint
                self._running -= 1
                self._cv.notify_all()
            fut._finish(value, error)

    def close(self, wait=True, timeout=None):
        """No more submissions; the queued jobs still run.  With a timeout
        (seconds), the jobs still queued when it runs out -- e.g. one whose
        footprint no longer fits beside the resident sessions -- finish
        with Rejected, and close returns once the running ones end."""
        with self._cv:
            self._closed = True
            self._cv.notify_all()
        if not wait:
            return
        t_end = None if timeout is None else time.perf_counter() + float(timeout)
        for t in self._workers:
            t.join(None if t_end is None else max(0.0, t_end - time.perf_counter()))
        if any(t.is_alive() for t in self._workers):
            with self._cv:
                while self._queue:
                    _, fut, _ = self._queue.popleft()
                    fut._finish(error=Rejected('scheduler closed before the request '
                                               'could be admitted'))
                self._cv.notify_all()
            for t in self._workers:
                t.join()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


def latency_summary(futures):
    """p50 / p99 / mean latency (s) and requests per second, over the
    requests that returned a result, from the first submit of one of them
    to the last completion; 'failed' counts the finished ones that raised
    (errors, cancelled, expired)."""
    ok = [f for f in futures if f.done() and f._error is None]
    failed = sum(1 for f in futures if f.done() and f._error is not None)
    lat = np.array([f.latency for f in ok])
    if not len(lat):
        return {'requests': 0, 'failed': failed}
    t0 = min(f.t_submit for f in ok)
    t1 = max(f.t_done for f in ok)
    q = np.array([f.queued for f in ok if f.queued is not None])
    return {'requests': int(len(lat)), 'failed': failed,
            'p50_s': float(np.percentile(lat, 50)),
            'p99_s': float(np.percentile(lat, 99)),
            'mean_s': float(lat.mean()),
            'queued_p50_s': float(np.percentile(q, 50)) if len(q) else None,
            'span_s': float(t1 - t0),
            'requests_per_s': float(len(lat) / (t1 - t0)) if t1 > t0 else None}


class _SharedLock:
    """Many holders in shared mode, or one in exclusive mode.  The server
    runs its host-side CUDA work (builds, session set-up and tear-down) in
    shared mode and CUDA-graph captures in exclusive mode: a capture must
    not overlap a device-wide synchronisation or allocation of another
    thread."""

    def __init__(self):
        self._cv = threading.Condition()
        self._shared = 0
        self._excl = False
        self._waiting_excl = 0

    def acquire_shared(self):
        with self._cv:
            # waiting exclusive holders go first (captures are rare and short)
            self._cv.wait_for(lambda: not self._excl and not self._waiting_excl)
            self._shared += 1

    def release_shared(self):
        with self._cv:
            self._shared -= 1
            self._cv.notify_all()

    def acquire_exclusive(self):
        with self._cv:
            self._waiting_excl += 1
            self._cv.wait_for(lambda: not self._excl and self._shared == 0)
            self._waiting_excl -= 1
            self._excl = True

    def release_exclusive(self):
        with self._cv:
            self._excl = False
            self._cv.notify_all()

    def shared(self):
        return _Held(self.acquire_shared, self.release_shared)

    def exclusive(self):
        return _Held(self.acquire_exclusive, self.release_exclusive)


class _Held:
    def __init__(self, acq, rel):
        self._acq, self._rel = acq, rel

    def __enter__(self):
        self._acq()
        return self

    def __exit__(self, *exc):
        self._rel()


class _Job:
    __slots__ = ('session', 'dm', 'footprint', 'key')

    def __init__(self, session, dm, footprint):
        self.session = session
        self.dm = dm
        self.footprint = footprint
        self.key = id(session)


class Session:
    """One molecule resident on the device: its engine (packed shell
    pairs) and grid.  Open through ExchangeServer.open_session."""

    def __init__(self, server, mol, coords, weights, omegas, tile_tol,
                 graphs=False):
        import torch
        from .cosx import CosxEngine
        self.server = server
        # graphs: the first build captures the session's build in a CUDA
        # graph (KBuildGraph) and later builds replay it
        self.graphs = bool(graphs)
        self.kgraph = None
        self.engine = CosxEngine(mol, device=server.device.index)
        self.coords = self.engine.relative(coords)
        self.weights = torch.as_tensor(np.ascontiguousarray(weights, dtype=np.float64),
                                       device=server.device)
        self.omegas = tuple(float(w) for w in omegas)
        self.tile_tol = float(tile_tol)
        self.nao = self.engine.nao
        self.npts = int(self.coords.shape[0])
        nom = len(self.omegas)
        kb = 8 * nom * self.nao * self.nao
        # running footprint: the build's workspace, D, K and its symmetrised
        # copy; resident: the pair tables are small next to the grid arrays
        self.footprint = (self.engine.workspace_bytes(self.npts) +
                          8 * self.nao * self.nao + 2 * kb)
        self.resident = 32 * self.npts + kb
        if self.graphs:
            # a captured build keeps its workspace and buffers for the
            # session's life: held as resident, not per request
            self.resident += self.footprint + kb
            self.footprint = 0
        self.closed = False

    def submit(self, dm, deadline=None):
        """One exchange build with density dm (nao, nao) FP64 (host):
        returns a Future whose result is K (len(omegas), nao, nao) FP64 on
        the host, symmetrised as the reference returns it.  deadline:
        seconds within which the build must start (else Expired); the
        Future's cancel() drops it while it waits."""
        return self.server._submit(self, dm, deadline)

    def close(self):
        if not self.closed:
            self.closed = True
            self.server._close_session(self)


class ExchangeServer:
    """Continuous-batching exchange builds on one GPU (module docstring).

    slots: builds in flight at once (one host thread + CUDA stream each).
    budget: device bytes for running builds + open sessions (default: 60 %
    of the free device memory at start-up).  gemm: the K build's GEMM mode.
    """

    def __init__(self, device=0, slots=4, budget=None, gemm='ozaki'):
        import torch
        self.device = torch.device('cuda', device if isinstance(device, int)
                                   else torch.device(device).index or 0)
        if budget is None:
            free, _ = torch.cuda.mem_get_info(self.device)
            budget = int(0.6 * free)
        self.gemm = gemm
        self._streams = [torch.cuda.Stream(device=self.device) for _ in range(slots)]
        self._sched = Scheduler(self._run, slots=slots, budget=budget)
        self._cuda = _SharedLock()
        self.futures = []

    @property
    def scheduler(self):
        return self._sched

    def open_session(self, mol, coords, weights, omegas=(0.0, 0.3), tile_tol=1e-11,
                     graphs=False):
        with self._cuda.shared():
            s = Session(self, mol, coords, weights, omegas, tile_tol, graphs)
        try:
            self._sched.reserve(s.resident, wait=True, headroom=s.footprint)
        except Rejected:
            with self._cuda.shared():
                s.engine.close()
            raise
        return s

    def _close_session(self, s):
        with self._cuda.shared():
            s.kgraph = None
            s.engine._ws = None
            s.engine.close()
        self._sched.release(s.resident)

    def _submit(self, session, dm, deadline=None):
        if session.closed:
            raise Rejected('session is closed')
        dm = np.ascontiguousarray(dm, dtype=np.float64)
        if dm.shape != (session.nao, session.nao):
            raise ValueError('dm must be (%d, %d)' % (session.nao, session.nao))
        fut = self._sched.submit(_Job(session, dm, session.footprint),
                                 deadline=deadline)
        self.futures.append(fut)
        return fut

    def _run(self, job, slot):
        import torch
        s = job.session
        eng = s.engine
        stream = self._streams[slot]
        nom = len(s.omegas)
        if s.graphs and s.kgraph is None:
            # the session keeps its workspace while its graph lives; the
            # capture (with its warm-up build) runs alone
            with self._cuda.exclusive(), torch.cuda.device(self.device), \
                    torch.cuda.stream(stream):
                s.kgraph = eng.capture_k_multi(s.coords, s.weights, s.omegas,
                                               tile_tol=s.tile_tol, gemm=self.gemm)
        with self._cuda.shared(), torch.cuda.device(self.device), \
                torch.cuda.stream(stream):
            dm_h = torch.from_numpy(job.dm).pin_memory()
            out = torch.empty((nom, s.nao, s.nao), dtype=torch.float64).pin_memory()
            if s.graphs:
                out.copy_(s.kgraph.run(dm_h), non_blocking=True)
            else:
                dm_d = torch.empty((s.nao, s.nao), dtype=torch.float64,
                                   device=self.device)
                dm_d.copy_(dm_h, non_blocking=True)
                K = eng.get_k_multi(s.coords, s.weights, dm_d, s.omegas,
                                    tile_tol=s.tile_tol, gemm=self.gemm, stats=False)
                out.copy_((K + K.transpose(1, 2)) * 0.5, non_blocking=True)
            done = torch.cuda.Event()
            done.record(stream)
            done.synchronize()
        if not s.graphs:
            # the workspace goes back to the allocator's cache for other builds
            eng._ws = None
        return out.numpy()

    def close(self):
        self._sched.close(wait=True)

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def summary(self):
        out = latency_summary(self.futures)
        out['slots'] = self._sched.slots
        out['budget_bytes'] = self._sched.budget
        out['max_concurrent'] = self._sched.max_running
        out['max_bytes_admitted'] = self._sched.max_used
        return out


class _ScfJob:
    """One SCF solve request (Scheduler job)."""

    def __init__(self, mol, footprint, reference_energy, precision, tag):
        self.mol = mol
        self.footprint = int(footprint)
        self.reference_energy = reference_energy
        self.precision = precision
        self.key = ('scf', tag)


# grid points per atom of this package's grids by level (Becke-partitioned
# atom grids; measured on water clusters and alkanes, rounded up)
_POINTS_PER_ATOM = {0: 1500, 1: 3100, 2: 5200, 3: 12000, 4: 24000}


class ScfServer:
    """Continuous batching of whole SCF solves on one GPU.

    A request is one molecule; its solve (DeviceRKS.kernel, the staged
    mixed form by default) keeps the density, the DIIS history, the grids
    and their AO values on the device from its first Fock build to the
    converged energy.  Requests that arrive while others run are admitted
    as soon as a slot and their device-memory footprint are free (the
    Scheduler: first fit in arrival order, one host thread and CUDA stream
    per slot), so the solves of different molecules overlap on the device.
    Every kernel of a solve has a fixed summation order and the solves
    synchronise their own streams only, so a molecule's energy is bitwise
    the same alone and in the mix.

    levels / coarse / stage_levels: the grids of every solve (as for
    DeviceRKS).  budget: device bytes for running solves (default 60 % of
    the free device memory at start-up)."""

    def __init__(self, device=0, slots=4, budget=None, levels=None, coarse=None,
                 stage_levels=None, k_tile_tol=1e-11):
        import torch
        self.device = torch.device('cuda', device if isinstance(device, int)
                                   else torch.device(device).index or 0)
        if budget is None:
            free, _ = torch.cuda.mem_get_info(self.device)
            budget = int(0.6 * free)
        self.levels, self.coarse, self.stage_levels = levels, coarse, stage_levels
        self.k_tile_tol = float(k_tile_tol)
        self._streams = [torch.cuda.Stream(device=self.device) for _ in range(slots)]
        self._sched = Scheduler(self._run, slots=slots, budget=budget)
        self._n = 0
        self.futures = []

    @property
    def scheduler(self):
        return self._sched

    def footprint(self, mol):
        """Device bytes of one solve (an upper estimate): the AO values of
        its XC and SGX grids and the deriv-1 values of its NLC grid (FP64),
        the exchange build's workspace (about 40 bytes per AO and SGX
        point) and the pair data."""
        from pyscf_wb97mv_fast_gb300.scf import DEFAULT_COARSE, DEFAULT_FINAL
        if self.stage_levels is not None:
            lv = {k: max(x for x in v if x is not None) if any(x is not None for x in v)
                  else None for k, v in self.stage_levels.items()}
        else:
            lv = dict(DEFAULT_FINAL, **(self.levels or {}))
        natm = int(mol.natm)
        pts = {k: (0 if v is None else _POINTS_PER_ATOM.get(int(v), 24000) * natm)
               for k, v in lv.items()}
        nao = int(mol.nao)
        xc_c = dict(DEFAULT_COARSE, **(self.coarse or {}))['xc']
        ao = 8 * nao * (pts['xc'] + pts['sgx'] + 4 * pts['nlc'] +
                        _POINTS_PER_ATOM.get(int(xc_c), 0) * natm)
        return ao + 40 * nao * pts['sgx'] + 64 * nao * nao + (64 << 20)

    def submit(self, mol, reference_energy=None, precision='mixed', deadline=None):
        """Queue the solve of mol (a Molecule); returns its Future, whose
        result() is the solve's summary (e_tot, converged, cycles, wall,
        error_vs_reference)."""
        from pyscf_wb97mv_fast_gb300.cosx import as_molecule
        mol = as_molecule(mol)
        self._n += 1
        fut = self._sched.submit(_ScfJob(mol, self.footprint(mol), reference_energy,
                                         precision, self._n), deadline=deadline)
        self.futures.append(fut)
        return fut

    def _run(self, job, slot):
        import torch
        from pyscf_wb97mv_fast_gb300.scf import DeviceRKS
        stream = self._streams[slot]
        with torch.cuda.device(self.device), torch.cuda.stream(stream):
            rks = DeviceRKS(job.mol, levels=self.levels, coarse=self.coarse,
                            stage_levels=self.stage_levels, k_tile_tol=self.k_tile_tol,
                            device=self.device.index)
            try:
                r = rks.kernel(precision=job.precision,
                               reference_energy=job.reference_energy)
            finally:
                rks.eng.close()
        out = {k: r.get(k) for k in ('e_tot', 'converged', 'cycles', 'wall',
                                     'error_vs_reference', 'precision')}
        out['nao'] = int(job.mol.nao)
        return out

    def close(self):
        self._sched.close(wait=True)

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def summary(self):
        out = latency_summary(self.futures)
        out['slots'] = self._sched.slots
        out['budget_bytes'] = self._sched.budget
        out['max_concurrent'] = self._sched.max_running
        out['max_bytes_admitted'] = self._sched.max_used
        return out


def poisson_arrivals(n, rate, seed):
    """n arrival times (s) of a Poisson process of the given rate."""
    rng = np.random.default_rng(seed)
    return np.cumsum(rng.exponential(1.0 / rate, size=n))


def replay(submit_fns, arrivals):
    """Calls submit_fns[i]() at arrivals[i] seconds after the start (real
    time, one thread); returns the futures in order."""
    t0 = time.perf_counter()
    futs = []
    for fn, t in zip(submit_fns, arrivals):
        dt = t0 + t - time.perf_counter()
        if dt > 0:
            time.sleep(dt)
        futs.append(fn())
    return futs


class Solve:
    """One SCF-shaped request: open a session for a molecule and run its
    exchange builds one after another (each cycle's density depends on the
    previous cycle's result in an SCF, so a solve's builds never overlap
    each other; different solves overlap freely).  run() returns the K of
    every cycle; t_arrival / t_done bracket the whole solve."""

    def __init__(self, server, mol, coords, weights, densities, omegas=(0.0, 0.3),
                 tile_tol=1e-11, tag=None, graphs=False):
        self.server = server
        self.graphs = graphs
        self.mol, self.coords, self.weights = mol, coords, weights
        self.densities = list(densities)
        self.omegas, self.tile_tol, self.tag = omegas, tile_tol, tag
        self.t_arrival = self.t_done = None
        self.results = None
        self.error = None
        self._thread = None

    def run(self):
        self.t_arrival = time.perf_counter()
        sess = self.server.open_session(self.mol, self.coords, self.weights,
                                        self.omegas, self.tile_tol, self.graphs)
        try:
            self.results = [sess.submit(dm).result() for dm in self.densities]
        finally:
            sess.close()
            self.t_done = time.perf_counter()
        return self.results

    def start(self):
        """run() on a client thread (errors kept in .error)."""
        def body():
            try:
                self.run()
            except BaseException as e:            # noqa: BLE001
                self.error = e
        self._thread = threading.Thread(target=body, daemon=True)
        self._thread.start()
        return self

    def join(self, timeout=None):
        self._thread.join(timeout)
        if self.error is not None:
            raise self.error
        return self.results

    @property
    def latency(self):
        return None if self.t_done is None else self.t_done - self.t_arrival


def solve_summary(solves):
    """Time-to-result of whole solves: p50 / p99 (s) and solves per second
    over the span from the first arrival to the last completion."""
    lat = np.array([s.latency for s in solves if s.latency is not None])
    if not len(lat):
        return {'solves': 0}
    t0 = min(s.t_arrival for s in solves)
    t1 = max(s.t_done for s in solves if s.t_done is not None)
    return {'solves': int(len(lat)), 'p50_s': float(np.percentile(lat, 50)),
            'p99_s': float(np.percentile(lat, 99)), 'mean_s': float(lat.mean()),
            'span_s': float(t1 - t0),
            'solves_per_s': float(len(lat) / (t1 - t0)) if t1 > t0 else None}
