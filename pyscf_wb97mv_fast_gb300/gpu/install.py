"""Install the GPU COSX path into a PySCF SCF object (reference:
pyscf_wb97mv_fast/gpu/install.py:209-336).

    hooks = install_gpu(mf, k=True)       # mf = dft.RKS(mol, xc='wb97m-v').COSX(pjs=True)
    try:
        e = mf.kernel()
    finally:
        hooks.restore_all()

k=True replaces the module function ``pyscf.sgx.sgx_jk.get_k_only`` with a
dispatcher: the SGX objects of this mf (``mf.with_df`` and the long-range
copies in ``mf.with_df._rsh_df``) go to ``GpuKBuilder`` (FP32 fused
kernels, screened with k_tile_tol, FP64 GEMMs); every other SGX object keeps
the original.  ``vv10=True`` (default) replaces ``mf._numint.nr_nlc_vxc`` by
the GPU VV10 flow.  ``overlap=True`` (default, as in the reference) wraps
``mf.get_veff`` so that the semilocal XC and VV10 flows run on a worker
thread, on their own CUDA stream, while this thread builds J and K with the
K flow on another stream (reference :138-206).

Deliberate contract change: no CPU fallback.  An error in a GPU flow of
this mf propagates (Unsupported, NativeError, DeviceOutOfMemory) -- after
the out-of-memory retry, which halves the grid tile twice like the
reference's _run_with_oom_retry (:99-109).  Importing this module does not
import PySCF; ``install_gpu`` does.
"""
import contextlib
import threading
import time

import numpy as np

from pyscf_wb97mv_fast_gb300.core.hooks import HookSet
from pyscf_wb97mv_fast_gb300.gpu import sgx_k as sgx_k_mod

DEFAULT_MEM_FRACTION = sgx_k_mod.DEFAULT_MEM_FRACTION


def is_oom(exc):
    """True when an exception is an out-of-memory condition."""
    if isinstance(exc, MemoryError):
        return True
    text = str(exc).lower()
    return 'out of memory' in text or 'cublas_status_alloc_failed' in text


def _run_with_oom_retry(flow, builder):
    """Run flow(builder); on out-of-memory halve the grid tile and retry,
    twice, then re-raise."""
    last = None
    b = builder
    for _ in range(3):
        try:
            return flow(b)
        except Exception as exc:                       # noqa: BLE001
            if not is_oom(exc):
                raise
            last = exc
            cur = b.blksize or getattr(b, 'last_tile', None) or (1 << 20)
            b = builder.with_blksize(max(32, int(cur) // 2))
    raise last


def flow_streams():
    """A factory of per-flow stream contexts: stream('k') / stream('xc')
    makes the calling thread's device work run on a private stream of that
    name (one per name and device, created on first use), after the work
    already queued on the thread's current stream.  device: the CUDA
    device (default: the calling thread's current one; a worker thread
    passes its caller's, since the current device is per thread).  Each flow then waits
    only for its own kernels when it reads a result back to the host, so
    the K build and the XC / VV10 flows overlap on the device.  Without a
    CUDA device it selects nothing: the flows themselves raise there."""
    streams = {}
    lock = threading.Lock()

    def stream(name, device=None):
        torch = sgx_k_mod._torch()
        if not torch.cuda.is_available():
            return contextlib.nullcontext()
        dev = torch.cuda.current_device() if device is None else int(device)
        with lock:
            s = streams.get((name, dev))
            if s is None:
                s = streams[(name, dev)] = torch.cuda.Stream(device=dev)
        s.wait_stream(torch.cuda.current_stream(dev))
        return torch.cuda.stream(s)
    return stream


_ABSENT = object()


def _current_device():
    """This thread's CUDA device, None without CUDA."""
    torch = sgx_k_mod._torch()
    return torch.cuda.current_device() if torch.cuda.is_available() else None


def _zero_xc(nao):
    """Stands in for nr_rks / nr_nlc_vxc while the stock get_veff builds J
    and K: no electrons, no energy, a zero potential."""
    def zero(*args, **kwargs):
        return 0, 0.0, np.zeros((nao, nao))
    return zero


def retag(like, arr, **override):
    """arr with the tags of like (PySCF's tag_array attributes: ecoul,
    exc, vj, vk), some of them replaced.  PySCF's lib.tag_array when PySCF
    imports, else a view of arr as like's array type."""
    tags = dict(getattr(like, '__dict__', {}))
    tags.update(override)
    try:
        from pyscf import lib
    except ImportError:
        out = np.asarray(arr).view(type(like))
        out.__dict__.update(tags)
        return out
    return lib.tag_array(arr, **tags)


def _overlap_factory(mf, ni, timings, stream):
    """mf.get_veff with the XC and VV10 flows on a worker thread.

    The stock get_veff runs on this thread with ni.nr_rks and
    ni.nr_nlc_vxc answering zero, so it builds J, K (through the K hook)
    and the Coulomb and exchange energies only; the worker computes exc and
    vxc of the same density meanwhile, and they are added afterwards (the
    same sums in another order).  The C-ABI calls and PySCF's J/K release
    the GIL, so both run at once.  Each call appends {'jk', 'xc', 'wait'}
    wall seconds to timings: J/K on this thread, XC + VV10 on the worker,
    and the wait for the worker after J/K.  A worker error is raised here.
    Densities the flows do not take (hermi=2, several densities) go to the
    stock get_veff unchanged."""
    def factory(orig):
        def get_veff(mol=None, dm=None, dm_last=None, vhf_last=None, hermi=1):
            if mol is None:
                mol = mf.mol
            if dm is None:
                dm = mf.make_rdm1()
            if hermi == 2 or not (isinstance(dm, np.ndarray) and dm.ndim == 2):
                return orig(mol, dm, dm_last, vhf_last, hermi)
            # the grids as the stock get_veff would set them up
            if mf.grids.coords is None:
                mf.initialize_grids(mol, dm)
            nlc = bool(mf.do_nlc())
            if nlc and mf.nlcgrids.coords is None:
                mf.nlcgrids.build(with_non0tab=True)
            nlc_code = None
            if nlc:
                nlc_code = mf.xc if ni.libxc.is_nlc(mf.xc) else mf.nlc
            xc_flow, nlc_flow = ni.nr_rks, ni.nr_nlc_vxc
            res = {}
            dev = _current_device()

            def worker():
                t0 = time.perf_counter()
                try:
                    with stream('xc', dev):
                        _, exc, vxc = xc_flow(mol, mf.grids, mf.xc, dm)
                        if nlc:
                            _, enlc, vnlc = nlc_flow(mol, mf.nlcgrids, nlc_code, dm)
                            exc = exc + enlc
                            vxc = vxc + vnlc
                    res['xc'] = (exc, vxc)
                except BaseException as err:           # noqa: BLE001
                    res['error'] = err
                res['t'] = time.perf_counter() - t0

            th = threading.Thread(target=worker, name='wb-xc', daemon=True)
            th.start()
            # the instance's own entries, put back exactly afterwards (a
            # method of the class shows through again)
            own = {n: vars(ni).get(n, _ABSENT) for n in ('nr_rks', 'nr_nlc_vxc')}
            zero = _zero_xc(dm.shape[0])
            ni.nr_rks = ni.nr_nlc_vxc = zero
            t0 = time.perf_counter()
            try:
                veff = orig(mol, dm, dm_last, vhf_last, hermi)
            finally:
                for n, v in own.items():
                    if v is _ABSENT:
                        delattr(ni, n)
                    else:
                        setattr(ni, n, v)
                t1 = time.perf_counter()
                th.join()
            timings.append({'jk': t1 - t0, 'xc': res.get('t'),
                            'wait': time.perf_counter() - t1})
            if 'error' in res:
                raise res['error']
            exc, vxc = res['xc']
            return retag(veff, np.asarray(veff) + vxc, exc=veff.exc + exc)
        return get_veff
    return factory


def check_scope(mol):
    """Raise Unsupported now, at install time, for a molecule the GPU
    flows do not take: a Cartesian basis, spinor shells, l above 3
    (Molecule.from_pyscf).  Host-only; the reference raises the same
    exception from its first K build (gpu/sgx_k.py:680-695)."""
    from pyscf_wb97mv_fast_gb300 import _native
    from pyscf_wb97mv_fast_gb300.cosx import as_molecule
    try:
        as_molecule(mol)
    except (ValueError, TypeError) as err:
        raise _native.Unsupported(_native.WB_ERR_UNSUPPORTED, str(err)) from err


def _sgx_jk_module():
    import pyscf.sgx.sgx_jk as mod
    return mod


def rsh_omegas(mf):
    """(0, omega) for a range-separated functional with omega > 0 and a
    full-range exchange part, (omega,) when only the long-range part is
    used, None otherwise or when the functional cannot be read
    (pyscf.dft.numint rsh_and_hybrid_coeff)."""
    try:
        ni = mf._numint
        omega, alpha, hyb = ni.rsh_and_hybrid_coeff(mf.xc, spin=mf.mol.spin)
    except Exception:
        return None
    omega = float(omega)
    if omega <= 0.0:
        return None
    if abs(float(hyb)) > 0.0:
        return (0.0, omega)
    return (omega,) if abs(float(alpha)) > 0.0 else None


def install_gpu(mf, backend=None, blksize=8192, vv10_tile_tol=0.0,
                functional_factory=None, verify_ao=True,
                gemm_dtype='float32', dtype='float32',
                mem_fraction=DEFAULT_MEM_FRACTION, overlap=True,
                semilocal=True, k=False, k_tile_tol=1e-11,
                openblas_threads=1, vv10=True, k_gemm='ozaki',
                sgx_jk_module=None, k_omegas='auto', k_precision='fp32'):
    """Hook the GPU flows into mf; returns a HookSet.

    The keywords and their defaults are the reference's
    (gpu/install.py:209-213): the XC and VV10 hooks always, the COSX K hook
    only with k=True.  backend must be None or 'cuda' (there is one
    backend).  blksize is the grid block of the semilocal XC flow (points
    per native call; None takes the whole grid); the K builder sizes its
    own grid tiles, as the reference's does.  gemm_dtype and dtype are
    accepted for the reference's 'float32' / 'float64' values: this flow's
    GEMMs take FP64 inputs whichever is asked (the X·D products are
    FP64-accurate and rounded once to FP32).  openblas_threads=1 holds a
    pthreads OpenBLAS to one thread until restore_all (None: leave it).
    semilocal=True replaces
    ``mf._numint.nr_rks`` by the GPU semilocal flow (gpu/xc.py), with
    functional_factory(xc_code, ni) -> XcFunctional (default: PySCF's
    libxc on the host).  sgx_jk_module lets tests pass a stand-in for
    pyscf.sgx.sgx_jk.  k_omegas (an addition): the omegas one SCF cycle
    asks K for with the same density, built together (GpuKBuilder
    omegas); 'auto' reads them from the range-separated functional of mf
    ((0, omega) when it has one), None builds one K per call.
    k_precision (an addition): 'fp32' (the mixed-precision K) or 'fp64'
    (the plain FP64 GPU form, for an FP64 tail on the GPU).  overlap=True
    wraps mf.get_veff (DFT objects only: mf.initialize_grids exists) to run
    the XC and VV10 flows beside J/K, and fills hooks.timings.
    """
    if backend not in (None, 'cuda', 'cupy'):
        raise ValueError("backend must be None or 'cuda'")
    for name, val in (('gemm_dtype', gemm_dtype), ('dtype', dtype)):
        if val not in ('float32', 'float64'):
            raise ValueError("%s must be 'float32' or 'float64'" % name)
    if getattr(mf, 'mol', None) is not None and (k or semilocal or vv10):
        check_scope(mf.mol)
    hooks = HookSet()
    if openblas_threads is not None:
        from pyscf_wb97mv_fast_gb300.core import blas_threads
        undo = blas_threads.limit_openblas_threads(openblas_threads)
        if undo is not None:
            hooks.on_restore(undo)      # registered first: undone last
    hooks.k_stats = []
    hooks.timings = []        # overlap: one {'jk', 'xc', 'wait'} per get_veff
    # overlap puts the K flow and the XC / VV10 flows on streams of their own
    stream = (flow_streams() if overlap
              else (lambda name, device=None: contextlib.nullcontext()))
    if k:
        mod = sgx_jk_module if sgx_jk_module is not None else _sgx_jk_module()
        holder = {}

        def k_factory(orig):
            def get_k_only(sgx, dm, hermi=1, direct_scf_tol=1e-13):
                df = mf.with_df
                rsh = getattr(df, '_rsh_df', None) or {}
                if not (sgx is df or any(sgx is v for v in rsh.values()
                                         if v is not None)):
                    return orig(sgx, dm, hermi, direct_scf_tol)
                b = holder.get('builder')
                if b is None:
                    oms = (rsh_omegas(mf) if isinstance(k_omegas, str)
                           and k_omegas == 'auto' else k_omegas)
                    b = sgx_k_mod.GpuKBuilder(mf.mol, tile_tol=k_tile_tol,
                                              gemm=k_gemm,
                                              precision=k_precision,
                                              omegas=oms)
                    b._build()
                    torch = sgx_k_mod._torch()
                    free, _ = torch.cuda.mem_get_info(b.engine.device)
                    b.mem_budget = int(free * mem_fraction)
                    holder['builder'] = b
                stats = {}

                def flow(bb):
                    kk = sgx_k_mod.get_k_only_gpu(bb, sgx, dm, hermi=hermi,
                                                  direct_scf_tol=direct_scf_tol)
                    stats.update(bb.last_stats)
                    return kk
                with stream('k'):
                    kk = _run_with_oom_retry(flow, b)
                hooks.k_stats.append(dict(stats))
                return kk
            return get_k_only

        hooks.wrap(mod, 'get_k_only', k_factory)
    if semilocal:
        ni = getattr(mf, '_numint', None)
        if ni is None:
            raise TypeError('mf has no _numint; not a DFT object?')
        from pyscf_wb97mv_fast_gb300.gpu import xc as xc_mod
        xctx = xc_mod.XcContext(mf.mol, functional_factory=functional_factory,
                                **({} if blksize is None
                                   else {'tile_pts': int(blksize)}))

        def rks_factory(orig):
            def nr_rks(mol, grids, xc_code, dms, relativity=0, hermi=1,
                       max_memory=2000, verbose=None):
                return xc_mod.gpu_nr_rks(xctx, ni, mol, grids, xc_code, dms,
                                         relativity, hermi, max_memory, verbose)
            return nr_rks
        hooks.wrap(ni, 'nr_rks', rks_factory)
    if vv10:
        ni = getattr(mf, '_numint', None)
        if ni is None:
            raise TypeError('mf has no _numint; not a DFT object?')
        from pyscf_wb97mv_fast_gb300.gpu import vv10 as vv10_mod
        ctx = vv10_mod.Vv10Context(mf.mol, tile_tol=vv10_tile_tol)

        def nlc_factory(orig):
            def nr_nlc_vxc(mol, grids, xc_code, dm, relativity=0, hermi=1,
                           max_memory=2000, verbose=None):
                return vv10_mod.gpu_nr_nlc_vxc(ctx, ni, mol, grids, xc_code, dm,
                                               relativity, hermi, max_memory,
                                               verbose)
            return nr_nlc_vxc
        hooks.wrap(ni, 'nr_nlc_vxc', nlc_factory)
    if overlap and hasattr(mf, 'initialize_grids'):
        ni = getattr(mf, '_numint', None)
        if ni is None:
            raise TypeError('mf has no _numint; not a DFT object?')
        hooks.wrap(mf, 'get_veff', _overlap_factory(mf, ni, hooks.timings, stream))
    return hooks


install = install_gpu
