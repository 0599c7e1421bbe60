"""Per-class kernel-variant autotuner of the fused G kernels.

Each shell-pair class has up to three kernel variants on a handle
(wb_cosx_set_class_variant): the two-omega kernel (both omegas of an SCF
cycle in one pass; staged records), the single-omega kernel with its
primitive-pair records staged in shared memory, and the single-omega
kernel with the records prefetched into registers.  Which is fastest
depends on the class's record sizes, its task count and the grid.  The
compiled-in defaults were measured on the water27 / def2-SVP workload.

autotune_classes times the whole G phase (wb_cosx_g_multi: block
statistics, the concurrent class kernels of both omegas and the
class-buffer sums, CUDA events on the launching stream) on the caller's
own grid and density, and walks the classes in decreasing work.  For each
class it tries the other available variants and keeps one only if it
beats the current phase time by `margin`.  The result is left set on the
engine.  Every variant is deterministic, and they agree to FP32 rounding.

The reference has one kernel per class (gpu/sgx_k.py:165-400) and no
tuner.
"""
import numpy as np

from pyscf_wb97mv_fast_gb300 import _native

def variant_name(v, nomega=2):
    """What runs for (dual, staged) in a call with nomega omegas: the
    two-omega kernel (always staged) in two-omega passes, else the
    single-omega kernel with staged or register-prefetched records."""
    dual, staged = v
    if dual and nomega == 2:
        return 'two-omega (staged)'
    return 'single-omega staged' if staged else 'single-omega register prefetch'


def candidates(cur, nomega=2):
    """The variants worth timing from the current one: two-omega passes
    only matter with two omegas."""
    if nomega == 2:
        return [(1, cur[1]), (0, 1), (0, 0)]
    return [(cur[0], 1), (cur[0], 0)]


def get_variant(eng, cls):
    d, s = _native.ctypes.c_int(0), _native.ctypes.c_int(0)
    _native.check(_native.lib().wb_cosx_get_class_variant(
        eng._h, int(cls), _native.ctypes.byref(d), _native.ctypes.byref(s)),
        'wb_cosx_get_class_variant')
    return int(d.value), int(s.value)


def set_variant(eng, cls, dual, staged):
    """True if the handle took the variant (False: the molecule cannot run
    it, the class keeps its variant)."""
    st = _native.lib().wb_cosx_set_class_variant(eng._h, int(cls), int(dual),
                                                 int(staged))
    if st == 0:
        return True
    if st == _native.WB_ERR_UNSUPPORTED:
        return False
    _native.check(st, 'wb_cosx_set_class_variant')
    return False


def time_g_phase(eng, coords_rel, weights, F, omegas, tile_tol, out, reps=3):
    """Best of reps G-phase times (ms) after one warm-up call."""
    torch = __import__('torch')
    eng.g_multi(coords_rel, weights, F, omegas, tile_tol, out=out, stats=False)
    best = float('inf')
    for _ in range(reps):
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record()
        eng.g_multi(coords_rel, weights, F, omegas, tile_tol, out=out, stats=False)
        e1.record()
        e1.synchronize()
        best = min(best, e0.elapsed_time(e1))
    return best


def autotune_classes(eng, coords_rel, weights, qd, omegas=(0.0, 0.3),
                     tile_tol=1e-11, reps=3, margin=0.01):
    """Tune the class variants of eng for this grid and density (device
    tensors as CosxEngine.get_k_multi takes them).  Returns a report:
    the G-phase time before and after, and per class the variant chosen
    and the times tried."""
    torch = __import__('torch')
    from pyscf_wb97mv_fast_gb300.cosx import round32
    X = eng.ao_eval(coords_rel)
    F = eng.ozaki_f(X, qd)
    del X
    out = torch.empty((len(omegas), eng.nao, round32(coords_rel.shape[0])),
                      dtype=torch.float32, device=eng.device)
    pairs = eng.pair_table()
    work = np.zeros(10)
    for row in pairs:
        work[int(row[4])] += float(row[7])
    classes = [int(c) for c in np.argsort(-work) if work[c] > 0]
    t0 = time_g_phase(eng, coords_rel, weights, F, omegas, tile_tol, out, reps)
    cur_t = t0
    report = {'g_ms_default': t0, 'classes': {}}
    nom = len(omegas)
    for c in classes:
        cur = get_variant(eng, c)
        tried = {variant_name(cur, nom): cur_t}
        best, best_t = cur, cur_t
        for v in candidates(cur, nom):
            if variant_name(v, nom) in tried:
                continue
            if not set_variant(eng, c, *v):
                continue
            t = time_g_phase(eng, coords_rel, weights, F, omegas, tile_tol, out, reps)
            tried[variant_name(v, nom)] = t
            if t < best_t * (1.0 - margin):
                best, best_t = v, t
        set_variant(eng, c, *best)
        cur_t = best_t
        report['classes'][int(c)] = {'chosen': variant_name(best, nom),
                                     'tried_ms': tried}
    report['g_ms_tuned'] = cur_t
    return report
