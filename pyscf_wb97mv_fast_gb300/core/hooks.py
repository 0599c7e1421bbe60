"""Reversible attribute patching (the reference's removable hook API,
pyscf_wb97mv_fast/core/hooks.py:26-107).

``HookSet.wrap(owner, name, factory)`` replaces ``owner.name`` by
``factory(original)`` and remembers how to undo it: an attribute defined on
the owner itself (module function, class attribute) is written back, one
that only shadowed a class-level attribute on an instance is deleted so the
class attribute shows through again.  ``restore_all()`` undoes every patch
and every ``on_restore`` callback in reverse order; a restored HookSet
refuses new patches.
"""

_ABSENT = object()


class HookSet:
    def __init__(self):
        self._undo = []
        self._closed = False

    def _check_open(self):
        if self._closed:
            raise RuntimeError('HookSet already restored')

    def wrap(self, owner, name, factory):
        """Replace owner.name by factory(orig); returns the undo record."""
        self._check_open()
        original = getattr(owner, name)
        own = (owner.__dict__.get(name, _ABSENT)
               if hasattr(owner, '__dict__') else _ABSENT)
        setattr(owner, name, factory(original))
        record = ('attr', owner, name, own)
        self._undo.append(record)
        return record

    def on_restore(self, fn):
        """Call fn() during restore_all(), in reverse order with the wraps."""
        self._check_open()
        self._undo.append(('call', fn))

    def restore_all(self):
        while self._undo:
            rec = self._undo.pop()
            if rec[0] == 'call':
                rec[1]()
                continue
            _, owner, name, own = rec
            if own is _ABSENT:
                delattr(owner, name)
            else:
                setattr(owner, name, own)
        self._closed = True

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.restore_all()


def reset_diis(mf_diis):
    """Drop the extrapolation history of a pyscf.lib.diis.DIIS in place,
    keeping its configuration (reference core/hooks.py:63-85).  None is a
    no-op."""
    if mf_diis is None:
        return
    mf_diis._buffer = {}
    mf_diis._bookkeep = []
    mf_diis._head = 0
    mf_diis._H = None
    mf_diis._xprev = None
    mf_diis._err_vec_touched = False
    mf_diis._diisfile = None


def track_residual(hooks, mf, sink):
    """Feed PySCF's per-cycle orbital-gradient norm envs['norm_gorb'] to
    sink(norm) through mf.callback, keeping any user callback."""
    def factory(prev):
        def callback(envs):
            sink(float(envs['norm_gorb']))
            if callable(prev):
                prev(envs)
        return callback
    return hooks.wrap(mf, 'callback', factory)
