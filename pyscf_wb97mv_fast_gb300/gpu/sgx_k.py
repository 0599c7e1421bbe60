"""GPU COSX exchange K behind the reference's builder interface.

``GpuKBuilder`` and ``get_k_only_gpu`` keep the names, arguments and
results of the reference (pyscf_wb97mv_fast/gpu/sgx_k.py:545-991): one
builder per molecule, ``get_k(sgx, dm, omega, hermi, direct_scf_tol)``
returns K (nao, nao) FP64 on the host for one RKS density matrix, with
``proj`` / ``sym`` read from the SGX object exactly as
``sgx_jk.get_k_only`` sets them up, and ``last_stats`` describing the call.

What runs underneath is the native library: one ``wb_cosx_get_k`` call per
K build does AO evaluation, F = fl32(X proj dm), the fused screen + G
kernels and K = X^T (w o G) on the device; the proj^T K and (K + K^T)/2
post-processing run on the device too, in FP64.

Contract changes (deliberate): there is no CPU fallback.  Inputs outside
the supported scope raise ``Unsupported`` (hermi != 1, several or
asymmetric density matrices, l > 3, ...); device failures raise
``NativeError`` / ``DeviceOutOfMemory``.  The install hook never calls the
CPU original for an mf it owns.
"""
import hashlib
import os
import time

import numpy as np

from pyscf_wb97mv_fast_gb300 import _native
from pyscf_wb97mv_fast_gb300.cosx import KSUB, CosxEngine, as_molecule

Unsupported = _native.Unsupported

LMAX = 3
_STATE_CACHE = 4           # grid states kept (full + LR copies alternate)
_BYTES_PER_POINT_NAO = 24  # workspace per point and AO: X64, F64/WG64, F, G
DEFAULT_MEM_FRACTION = 0.6


def _torch():
    import torch
    return torch


class _GridState:
    """Device copies of one grids object's coordinates (kernel frame) and
    weights, plus the tile size (points per native call)."""

    def __init__(self, builder, grids):
        torch = _torch()
        coords = np.asarray(grids.coords, dtype=np.float64)
        weights = np.asarray(grids.weights, dtype=np.float64)
        self.ngrids = coords.shape[0]
        eng = builder.engine
        self.coords = eng.relative(coords)
        self.weights = torch.as_tensor(weights, dtype=torch.float64,
                                       device=eng.device).contiguous()
        self.grids_id = id(grids)
        # content fingerprint: copies of one grid (e.g. the range-separated
        # SGX objects of one mf) are recognised as the same grid
        h = hashlib.blake2b(digest_size=16)
        h.update(np.ascontiguousarray(coords).tobytes())
        h.update(np.ascontiguousarray(weights).tobytes())
        self.fingerprint = h.hexdigest()


class GpuKBuilder:
    """Per-molecule COSX K builder on one CUDA device (reference:
    GpuKBuilder, gpu/sgx_k.py:545-851).

    tile_tol: screening threshold (1e-11 default, 0 keeps every task).
    blksize: grid points per native call (None: as many as the memory
    budget allows; the reference tiles by SMs x 32 warps x 32 points
    because its target cards have 8-24 GB).
    gemm: 'ozaki' (FP64-accurate split on the bf16 tensor cores, default),
    'native' (cuBLAS DGEMM) or 'emulated' (cuBLAS FP64 emulation).
    omegas: the range-separation parameters one SCF cycle asks for with
    the same density (e.g. (0.0, 0.3) for wB97M-V: full-range and
    long-range K).  When get_k is called for one of them, all are built in
    one native call (AO values and F shared) and the others are kept until
    asked for with the same density, grid and projector; any other call
    drops them.  None (default): one K per call.
    precision (an addition): 'fp32' (default: the fused FP32 G kernels,
    F rounded once to FP32) or 'fp64' (the plain FP64 form,
    wb_cosx_get_k_fp64: FP64 F, FP64 G kernels, DGEMMs; the whole grid in
    one call) -- the operator of an FP64 tail on the GPU.
    """

    def __init__(self, mol, device=None, tile_tol=1e-11, mem_budget=None,
                 origin=None, blksize=None, gemm='ozaki', omegas=None,
                 precision='fp32'):
        self.mol = mol
        self.tile_tol = float(tile_tol)
        self.origin = origin
        self.device = device
        self.mem_budget = mem_budget
        self.blksize = None if blksize is None else int(blksize)
        if gemm not in ('ozaki', 'native', 'emulated'):
            raise ValueError("gemm must be 'ozaki', 'native' or 'emulated'")
        self.gemm = gemm
        self.omegas = None if omegas is None else tuple(float(w) for w in omegas)
        if precision not in ('fp32', 'fp64'):
            raise ValueError("precision must be 'fp32' or 'fp64'")
        self.precision = precision
        self._pending = None       # (key, dm copy, {omega: K host}) of a multi build
        self.engine = None
        self._grids_states = {}
        self.last_stats = {}
        self._built = False

    def _build(self):
        if self._built:
            return
        torch = _torch()
        if not torch.cuda.is_available():
            raise _native.NativeError(_native.WB_ERR_NO_DEVICE,
                                      'GpuKBuilder needs a CUDA device')
        self.engine = CosxEngine(as_molecule(self.mol), origin=self.origin,
                                 device=self.device)
        self.nao = self.engine.nao
        if self.mem_budget is None:
            free, _ = torch.cuda.mem_get_info(self.engine.device)
            self.mem_budget = int(free * DEFAULT_MEM_FRACTION)
        self._built = True

    def with_blksize(self, blksize):
        """Clone sharing every cache; only the tile size changes (the OOM
        lever, halved by install._run_with_oom_retry)."""
        self._build()
        clone = GpuKBuilder.__new__(GpuKBuilder)
        clone.__dict__.update(self.__dict__)
        clone.blksize = int(blksize)
        return clone

    def _tile(self, npts):
        """Points per native call (0 = all of them in one tile)."""
        if self.blksize is not None:
            t = max(KSUB, self.blksize // KSUB * KSUB)
        else:
            per_pt = _BYTES_PER_POINT_NAO * max(self.nao, 1) + 64
            t = max(KSUB, int(self.mem_budget // per_pt) // KSUB * KSUB)
        self.last_tile = min(t, max(KSUB, npts))
        return 0 if t >= npts else t

    def _grid_state(self, grids):
        key = (id(grids), int(np.asarray(grids.weights).size))
        st = self._grids_states.get(key)
        if st is None:
            st = _GridState(self, grids)
            self._grids_states[key] = st
            while len(self._grids_states) > _STATE_CACHE:
                self._grids_states.pop(next(iter(self._grids_states)))
        return st

    def get_k(self, sgx, dm, omega, hermi=1, direct_scf_tol=1e-13):
        """K (nao, nao) FP64 host for one RKS density matrix on sgx's grid.
        With PYSCF_WB97MV_KPROFILE=1 each phase ends with a synchronisation
        of the flow's stream and last_stats['phases'] holds its seconds
        (checks, build, pjs, grid_state, proj_dm, kernel, post, to_host),
        with the device phases of the kernel call in last_stats['phase_ms']
        (reference gpu/sgx_k.py:667-679)."""
        t0 = time.perf_counter()
        torch = _torch()
        lap = _Laps(torch) if profiling_enabled() else None
        if hermi != 1:
            raise Unsupported(_native.WB_ERR_UNSUPPORTED,
                              'GPU COSX K supports hermi=1 only')
        dm = np.asarray(dm)
        if dm.ndim != 2 or dm.shape[0] != dm.shape[1]:
            raise Unsupported(_native.WB_ERR_UNSUPPORTED,
                              'GPU COSX K supports a single square density matrix')
        if not np.allclose(dm, dm.T, rtol=0, atol=1e-12):
            raise Unsupported(_native.WB_ERR_UNSUPPORTED,
                              'GPU COSX K needs a symmetric density matrix')
        if lap:
            lap('checks')
        self._build()
        if lap:
            lap('build')
        if dm.shape[0] != self.nao:
            raise Unsupported(_native.WB_ERR_UNSUPPORTED,
                              'dm does not match the molecule')
        mol = sgx.mol
        grids = sgx.grids
        pjs = getattr(sgx, '_pjs_data', None)
        if (pjs is None or getattr(pjs, 'mol', mol) is not mol
                or getattr(pjs, 'grids', grids) is not grids
                or getattr(pjs, '_itol', direct_scf_tol) != direct_scf_tol):
            sgx._build_pjs(direct_scf_tol)
            pjs = sgx._pjs_data
        proj = np.asarray(pjs._overlap_correction_matrix, dtype=np.float64)
        sym = bool(pjs.sym_ovlp)
        if lap:
            lap('pjs')
        state = self._grid_state(grids)
        if lap:
            lap('grid_state')
        key = (state.fingerprint, sym, self.tile_tol, self.gemm, self.precision)
        omega = float(omega)
        hit = self._take_pending(key, dm, proj, omega)
        if hit is not None:
            st = dict(self.last_stats)
            st['wall'] = time.perf_counter() - t0
            st['kernel'] = 0.0
            st['from_multi'] = True
            self.last_stats = st
            return hit
        dev = self.engine.device
        proj_d = torch.as_tensor(proj, device=dev)
        qd = proj_d @ torch.as_tensor(dm, dtype=torch.float64, device=dev)
        if lap:
            lap('proj_dm')
        tk0 = time.perf_counter()
        multi = self.omegas is not None and omega in self.omegas and len(self.omegas) > 1
        if self.precision == 'fp64':
            Ks = self.engine.get_k_fp64(state.coords, state.weights, qd,
                                        self.omegas if multi else (omega,),
                                        tile_tol=self.tile_tol)
        elif multi:
            Ks = self.engine.get_k_multi(state.coords, state.weights, qd,
                                         self.omegas, tile_tol=self.tile_tol,
                                         tile_pts=self._tile(state.ngrids),
                                         gemm=self.gemm, profile=bool(lap))
        else:
            Ks = self.engine.get_k(state.coords, state.weights, qd, omega,
                                   tile_tol=self.tile_tol,
                                   tile_pts=self._tile(state.ngrids),
                                   gemm=self.gemm, profile=bool(lap))[None]
        if lap:
            lap('kernel')
        if sym:
            Ks = proj_d.T[None] @ Ks
        Ks = (Ks + Ks.transpose(1, 2)) * 0.5
        if lap:
            lap('post')
        Kh = Ks.cpu().numpy()
        if lap:
            lap('to_host')
        if multi:
            done = {w: Kh[j] for j, w in enumerate(self.omegas) if w != omega}
            self._pending = (key, dm.copy(), proj.copy(), done)
            Kh = Kh[self.omegas.index(omega)]
        else:
            self._pending = None
            Kh = Kh[0]
        st = dict(self.engine.last_stats)
        st['wall'] = time.perf_counter() - t0
        st['kernel'] = time.perf_counter() - tk0
        st['from_multi'] = False
        if lap:
            st['phases'] = lap.phases
        self.last_stats = st
        return Kh

    def _take_pending(self, key, dm, proj, omega):
        """A K of the last multi-omega build for this density, grid and
        projector, or None (the pending set is dropped on any miss)."""
        pend = self._pending
        if pend is None:
            return None
        pkey, pdm, pproj, done = pend
        if (pkey != key or omega not in done or pdm.shape != dm.shape
                or not np.array_equal(pdm, dm) or pproj.shape != proj.shape
                or not np.array_equal(pproj, proj)):
            self._pending = None
            return None
        K = done.pop(omega)
        if not done:
            self._pending = None
        return K

    def kernel_info(self):
        """Per task class: pairs and primitive pairs of this molecule."""
        self._build()
        names = ['l%d%d' % (la, lb) for la in range(LMAX + 1)
                 for lb in range(la + 1)]
        return {n: (self.engine.class_pairs[i], self.engine.class_prim_pairs[i])
                for i, n in enumerate(names)}


def get_k_only_gpu(builder, sgx, dm, hermi=1, direct_scf_tol=1e-13):
    """Same signature/contract as pyscf.sgx.sgx_jk.get_k_only for one RKS
    dm; omega is read from sgx.mol.omega (reference gpu/sgx_k.py:983-991)."""
    omega = float(getattr(sgx.mol, 'omega', 0.0) or 0.0)
    return builder.get_k(sgx, dm, omega, hermi=hermi,
                         direct_scf_tol=direct_scf_tol)


class PjsData:
    """The two attributes of PySCF's SGX PJS data the K build reads."""

    def __init__(self, mol, grids, proj, sym=False, itol=1e-13):
        self.mol = mol
        self.grids = grids
        self._overlap_correction_matrix = proj
        self.sym_ovlp = sym
        self._itol = itol


class SyntheticSGX:
    """Stand-in for PySCF's SGX object when PySCF is absent: ``mol``,
    ``grids`` and the PJS data (proj = identity unless given)."""

    def __init__(self, mol, grids, proj=None, sym=False):
        self.mol = mol
        self.grids = grids
        self._proj = proj
        self._sym = sym
        self._pjs_data = None

    def _build_pjs(self, direct_scf_tol=1e-13):
        nao = self.mol.nao
        proj = np.eye(nao) if self._proj is None else np.asarray(self._proj)
        self._pjs_data = PjsData(self.mol, self.grids, proj, self._sym,
                                 direct_scf_tol)


def profiling_enabled():
    return os.environ.get('PYSCF_WB97MV_KPROFILE') == '1'


class _Laps:
    """lap(name): synchronise this thread's current CUDA stream and book the
    seconds since the previous lap under name (phase timing of get_k)."""

    def __init__(self, torch):
        self._torch = torch
        self.phases = {}
        self._t = time.perf_counter()

    def _sync(self):
        if self._torch.cuda.is_available():
            self._torch.cuda.current_stream().synchronize()

    def __call__(self, name):
        self._sync()
        t = time.perf_counter()
        self.phases[name] = self.phases.get(name, 0.0) + (t - self._t)
        self._t = t
