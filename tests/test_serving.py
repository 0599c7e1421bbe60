"""The continuous-batching scheduler (serving.Scheduler) on the CPU: slots,
memory budget, first-fit admission, per-session order, errors.  The GPU
executor is covered by tests/test_gpu_serving.py."""
import threading
import time

import numpy as np
import pytest

from pyscf_wb97mv_fast_gb300.serving import (Rejected, Scheduler, latency_summary,
                                             poisson_arrivals, replay)


class Job:
    def __init__(self, name, footprint, key, dur=0.02):
        self.name, self.footprint, self.key, self.dur = name, footprint, key, dur


class Recorder:
    def __init__(self):
        self.lock = threading.Lock()
        self.running = {}
        self.max_running = 0
        self.max_bytes = 0
        self.order = []
        self.overlaps = []

    def __call__(self, job, slot):
        with self.lock:
            for other in self.running.values():
                assert other.key != job.key, 'two jobs of one key at once'
            self.running[job.name] = job
            self.max_running = max(self.max_running, len(self.running))
            self.max_bytes = max(self.max_bytes,
                                 sum(j.footprint for j in self.running.values()))
            self.order.append(job.name)
        time.sleep(job.dur)
        with self.lock:
            del self.running[job.name]
        return job.name, slot


def test_slots_and_budget_are_never_exceeded():
    rec = Recorder()
    s = Scheduler(rec, slots=3, budget=100)
    futs = [s.submit(Job('j%d' % i, 30 + (i % 3) * 10, key=i)) for i in range(24)]
    s.close()
    assert [f.result()[0] for f in futs] == ['j%d' % i for i in range(24)]
    assert rec.max_running <= 3
    assert rec.max_bytes <= 100
    assert rec.max_running >= 2            # work did overlap
    assert s.max_running == rec.max_running


def test_first_fit_lets_small_jobs_pass_a_large_one():
    rec = Recorder()
    s = Scheduler(rec, slots=4, budget=100)
    a = s.submit(Job('a', 60, key='a', dur=0.2))
    time.sleep(0.05)                       # a is running
    big = s.submit(Job('big', 80, key='big', dur=0.01))   # waits for a
    small = s.submit(Job('small', 30, key='small', dur=0.01))
    small.result(5)
    assert not big.done()                  # small passed big
    s.close()
    assert big.result() and a.result()
    assert rec.order.index('small') < rec.order.index('big')


def test_jobs_of_one_key_run_in_submission_order():
    rec = Recorder()
    s = Scheduler(rec, slots=4, budget=None)
    futs = [s.submit(Job('s%d' % i, 1, key='same', dur=0.005)) for i in range(10)]
    futs += [s.submit(Job('o%d' % i, 1, key='o%d' % i, dur=0.005)) for i in range(5)]
    s.close()
    for f in futs:
        f.result()
    same = [n for n in rec.order if n.startswith('s')]
    assert same == ['s%d' % i for i in range(10)]


def test_rejections_and_errors():
    def boom(job, slot):
        raise RuntimeError('kernel failed: ' + job.name)
    s = Scheduler(boom, slots=2, budget=50)
    with pytest.raises(Rejected):
        s.submit(Job('huge', 51, key=1))
    s.reserve(20)
    with pytest.raises(Rejected):
        s.submit(Job('now too big', 40, key=2))
    with pytest.raises(Rejected):
        s.reserve(40)
    f = s.submit(Job('x', 10, key=3))
    with pytest.raises(RuntimeError, match='kernel failed: x'):
        f.result(5)
    s.release(20)
    s.close()
    with pytest.raises(Rejected):
        s.submit(Job('late', 1, key=4))
    with pytest.raises(ValueError):
        Scheduler(boom, slots=0)


def test_resident_bytes_count_against_admission():
    rec = Recorder()
    s = Scheduler(rec, slots=4, budget=100)
    s.reserve(50)
    futs = [s.submit(Job('j%d' % i, 25, key=i, dur=0.03)) for i in range(6)]
    for f in futs:
        f.result(5)
    assert rec.max_bytes <= 50             # two jobs at a time next to 50 resident
    assert s.max_used <= 100
    s.close()


def test_latency_summary_and_arrivals():
    a = poisson_arrivals(200, rate=50.0, seed=3)
    b = poisson_arrivals(200, rate=50.0, seed=3)
    assert np.array_equal(a, b) and np.all(np.diff(a) > 0)
    assert 2.5 < a[-1] < 6.0               # 200 arrivals at 50/s
    s = Scheduler(lambda job, slot: job.name, slots=2)
    jobs = [Job('r%d' % i, 1, key=i, dur=0) for i in range(8)]
    futs = replay([lambda j=j: s.submit(j) for j in jobs],
                  np.linspace(0.0, 0.07, 8))
    s.close()
    summ = latency_summary(futs)
    assert summ['requests'] == 8
    assert 0 <= summ['p50_s'] <= summ['p99_s']
    assert summ['span_s'] >= 0.07
    assert latency_summary([])['requests'] == 0


def test_reserve_waits_for_room():
    rec = Recorder()
    s = Scheduler(rec, slots=2, budget=100)
    f = s.submit(Job('long', 70, key='a', dur=0.2))
    time.sleep(0.05)                       # 70 bytes running
    t0 = time.perf_counter()
    s.reserve(50, wait=True, timeout=5)    # waits for the job to end
    assert time.perf_counter() - t0 > 0.05 and f.done()
    with pytest.raises(Rejected):
        s.reserve(60, wait=True, timeout=0.05)   # 50 + 60 > 100, nothing ends
    with pytest.raises(Rejected):
        s.reserve(101, wait=True)                # above the whole budget
    s.release(50)
    s.close()


def test_session_headroom_prevents_starvation():
    """Sessions hold resident bytes while their requests queue.  Admitting
    a session only with room for its own request on top (headroom) keeps
    the most recent session runnable: here three sessions of 20 resident +
    50 per request share a budget of 100; without headroom the third
    admission (60 resident) would leave no room for any request."""
    rec = Recorder()
    s = Scheduler(rec, slots=4, budget=100)
    done = []

    def session(name):
        s.reserve(20, wait=True, timeout=10, headroom=50)
        try:
            for i in range(2):
                s.submit(Job('%s%d' % (name, i), 50, key=name, dur=0.02)).result(10)
        finally:
            s.release(20)
        done.append(name)

    ts = [threading.Thread(target=session, args=(n,)) for n in 'abc']
    for t in ts:
        t.start()
    for t in ts:
        t.join(20)
    assert sorted(done) == ['a', 'b', 'c']
    assert s.max_used <= 100 and s.resident == 0
    with pytest.raises(Rejected):
        s.reserve(60, wait=True, headroom=50)       # can never fit
    s.close()


def test_cancel_drops_a_waiting_request_only():
    """A queued request can be cancelled; a running or finished one
    cannot.  One slot: the first job runs while the others wait."""
    from pyscf_wb97mv_fast_gb300.serving import Cancelled
    rec = Recorder()
    s = Scheduler(rec, slots=1, budget=None)
    f1 = s.submit(Job('a', 1, key='a', dur=0.2))
    time.sleep(0.05)
    f2 = s.submit(Job('b', 1, key='b', dur=0.01))
    f3 = s.submit(Job('c', 1, key='c', dur=0.01))
    assert not f1.cancel()                        # running
    assert f2.cancel() and not f2.cancel()        # waiting, then gone
    with pytest.raises(Cancelled):
        f2.result(1)
    assert f3.result(5) == ('c', 0) and f1.result(5) == ('a', 0)
    assert not f3.cancel()                        # finished
    assert rec.order == ['a', 'c']
    summ = latency_summary([f1, f2, f3])          # the cancelled one failed
    assert summ['requests'] == 2 and summ['failed'] == 1
    s.close()


def test_deadline_expires_requests_that_cannot_start_in_time():
    """Requests whose deadline passes while the budget is held are
    dropped with Expired, and the idle slots wake for the deadline without
    any other event; one that starts in time runs."""
    from pyscf_wb97mv_fast_gb300.serving import Expired
    rec = Recorder()
    s = Scheduler(rec, slots=3, budget=100)
    big = s.submit(Job('big', 90, key='big', dur=1.0))
    time.sleep(0.05)
    late = s.submit(Job('late', 50, key='late'), deadline=0.1)
    ok = s.submit(Job('ok', 50, key='ok'), deadline=5.0)
    t0 = time.perf_counter()
    with pytest.raises(Expired):
        late.result(5)
    assert time.perf_counter() - t0 < 0.6         # at its deadline, not at big's end
    assert ok.result(5)[0] == 'ok'
    big.result(5)
    assert 'late' not in rec.order and s.max_used <= 100
    s.close()


def test_allocation_failure_frees_its_slot_and_budget():
    """A build whose device allocation fails (a fake DeviceOutOfMemory from
    the run function) hands the error to its request and gives its slot
    and bytes back: the next request, which needs the whole budget, runs."""
    from pyscf_wb97mv_fast_gb300._native import DeviceOutOfMemory, WB_ERR_OUT_OF_MEMORY

    def run(job, slot):
        if job.name == 'oom':
            raise DeviceOutOfMemory(WB_ERR_OUT_OF_MEMORY, 'cudaMallocAsync: out of memory')
        return job.name

    s = Scheduler(run, slots=1, budget=100)
    f = s.submit(Job('oom', 100, key='a'))
    g = s.submit(Job('next', 100, key='b'))
    with pytest.raises(MemoryError, match='out of memory'):
        f.result(5)
    assert g.result(5) == 'next'
    s.close()
    assert s._used == 0 and s._running == 0 and s.max_used <= 100


def test_scheduler_invariants_on_random_mixes():
    """Random job mixes (footprints, sessions, durations, slot counts,
    budgets): the budget and the slot count are never exceeded, each
    session's jobs run one at a time in submission order, and every job
    finishes."""
    hyp = pytest.importorskip('hypothesis')
    st = pytest.importorskip('hypothesis.strategies')

    @hyp.settings(max_examples=60, deadline=None)
    @hyp.given(slots=st.integers(1, 4), budget=st.integers(10, 60),
               jobs=st.lists(st.tuples(st.integers(1, 10), st.integers(0, 3),
                                       st.sampled_from([0.0, 0.001, 0.003])),
                             min_size=1, max_size=14))
    def check(slots, budget, jobs):
        rec = Recorder()
        s = Scheduler(rec, slots=slots, budget=budget)
        futs = [s.submit(Job('j%d' % i, fp, key=k, dur=d))
                for i, (fp, k, d) in enumerate(jobs)]
        for f in futs:
            f.result(10)
        s.close()
        assert rec.max_running <= slots and rec.max_bytes <= budget
        assert s.max_used <= budget and s._used == 0
        for k in set(k for _, k, _ in jobs):
            mine = ['j%d' % i for i, (_, kk, _) in enumerate(jobs) if kk == k]
            assert [n for n in rec.order if n in mine] == mine

    check()


def test_close_with_timeout_rejects_a_job_that_can_never_fit():
    """A queued job that fit when it was submitted, but no longer does
    beside sessions reserved later, cannot block close() for ever: with a
    timeout it finishes with Rejected."""
    gate = threading.Event()

    def run(job, slot):
        if job.name == 'b':
            gate.wait(5.0)
        return job.name

    s = Scheduler(run, slots=2, budget=100)
    s.reserve(40)                                   # session A
    fb = s.submit(Job('b', 50, 'b'))                # runs: 90 of 100
    time.sleep(0.05)
    fa = s.submit(Job('a', 50, 'a'))                # fits at submit, waits for b
    s.reserve(20)                                   # session C: 60 resident
    gate.set()                                      # b ends; a needs 110 > 100
    t0 = time.perf_counter()
    s.close(timeout=0.3)
    assert time.perf_counter() - t0 < 3.0
    assert fb.result(timeout=1.0) == 'b'
    with pytest.raises(Rejected):
        fa.result(timeout=1.0)


def test_scheduler_as_context_manager_runs_queued_jobs_then_stops():
    """Leaving a with-block closes the scheduler: the jobs queued in it
    still run to the end, its workers stop, and it takes no new request."""
    def run(job, slot):
        time.sleep(0.01)
        return job.name

    with Scheduler(run, slots=2, budget=100) as s:
        futs = [s.submit(Job(str(i), 30, str(i))) for i in range(6)]
    assert [f.result(timeout=0) for f in futs] == [str(i) for i in range(6)]
    assert not any(t.is_alive() for t in s._workers)
    with pytest.raises(Rejected):
        s.submit(Job('late', 10, 'late'))


def test_latency_span_starts_at_the_first_successful_request():
    class F:
        def __init__(self, t_submit, t_done, error=None):
            self.t_submit, self.t_done, self._error = t_submit, t_done, error
            self.t_start = t_submit
            self.latency = t_done - t_submit
            self.queued = 0.0

        def done(self):
            return True
    futs = [F(0.0, 0.5, error=RuntimeError('cancelled')), F(10.0, 11.0), F(10.5, 12.0)]
    out = latency_summary(futs)
    assert out['requests'] == 2 and out['failed'] == 1
    assert out['span_s'] == pytest.approx(2.0)
