"""Hold a threaded OpenBLAS to a fixed thread count while the hooks are on
(reference: pyscf_wb97mv_fast/core/blas_threads.py:89-108, the
``openblas_threads`` keyword of install_gpu).

PySCF calls BLAS from inside its own OpenMP regions.  A pthreads OpenBLAS
then starts its own threads on top of OpenMP's and oversubscribes the host
cores.  ``OPENBLAS_NUM_THREADS`` only acts before the library is loaded, so
the limit is set through the library's exported setter, and undone by the
HookSet.

Rules (the reference's):
* a process whose user set ``OPENBLAS_NUM_THREADS`` or ``GOTO_NUM_THREADS``
  is left alone;
* only libraries built with pthreads threading (``get_parallel() == 1``)
  are touched; sequential and OpenMP builds are not;
* each distinct library is changed once, even when several mapped files
  re-export the same setter.

Nothing here touches the GPU.
"""
import collections
import ctypes
import os

ENV_OVERRIDES = ('OPENBLAS_NUM_THREADS', 'GOTO_NUM_THREADS')

# exported-name patterns of OpenBLAS builds: the plain library and the
# scipy-openblas wheels (with and without the ILP64 suffix)
_SYMBOL_FORMS = ('openblas_{}', 'scipy_openblas_{}64_', 'scipy_openblas_{}')

BlasLib = collections.namedtuple('BlasLib', 'path parallel get_threads set_threads')


def _open_mapped(path):
    """The already-mapped library at path (never loads a new one)."""
    mode = getattr(os, 'RTLD_NOLOAD', 0) | getattr(os, 'RTLD_LOCAL', 0)
    try:
        return ctypes.CDLL(path, mode=mode)
    except OSError:
        return None


def _functions(cdll):
    for form in _SYMBOL_FORMS:
        try:
            par = getattr(cdll, form.format('get_parallel'))
            get = getattr(cdll, form.format('get_num_threads'))
            put = getattr(cdll, form.format('set_num_threads'))
        except AttributeError:
            continue
        for f in (par, get):
            f.restype, f.argtypes = ctypes.c_int, []
        put.restype, put.argtypes = None, [ctypes.c_int]
        return par, get, put
    return None


def mapped_blas_libraries(maps_path='/proc/self/maps'):
    """BlasLib entries for every OpenBLAS mapped into this process, one per
    distinct setter (Linux; an empty list elsewhere)."""
    try:
        with open(maps_path) as fh:
            files = {ln.split()[-1] for ln in fh
                     if ln.rstrip().endswith('.so') or '.so.' in ln}
    except OSError:
        return []
    libs, setters = [], set()
    for path in sorted(files):
        if 'blas' not in os.path.basename(path).lower():
            continue
        cdll = _open_mapped(path)
        fns = _functions(cdll) if cdll is not None else None
        if fns is None:
            continue
        key = ctypes.cast(fns[2], ctypes.c_void_p).value
        if key in setters:
            continue
        setters.add(key)
        libs.append(BlasLib(path, *fns))
    return libs


def limit_openblas_threads(n=1, libs=None, environ=None):
    """Set every pthreads OpenBLAS to n threads.

    Returns a callable that puts the previous counts back, or None when
    nothing was changed (user override in the environment, or no pthreads
    OpenBLAS mapped).  ``libs`` and ``environ`` let tests pass stand-ins.
    """
    env = os.environ if environ is None else environ
    if any(env.get(k) for k in ENV_OVERRIDES):
        return None
    if libs is None:
        libs = mapped_blas_libraries()
    changed = []
    for lib in libs:
        if int(lib.parallel()) != 1:
            continue
        changed.append((lib, int(lib.get_threads())))
        lib.set_threads(int(n))
    if not changed:
        return None

    def restore():
        for lib, before in reversed(changed):
            lib.set_threads(before)
    return restore
