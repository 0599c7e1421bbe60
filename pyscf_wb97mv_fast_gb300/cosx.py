"""CosxEngine: one native COSX handle (molecule x device) driven from PyTorch.

Device buffers are torch tensors; every call passes raw pointers and the
current torch stream through the C ABI (``_native``).  The engine owns the
packed shell-pair tables (uploaded once per molecule) and a cached device
workspace; it never copies data to the host except the final K and, when
asked for, the counters of the last call.
"""
import numpy as np

from pyscf_wb97mv_fast_gb300 import _native
from pyscf_wb97mv_fast_gb300.basis import Molecule

KSUB = 32          # grid points per sub-block = one warp


def _torch():
    import torch
    return torch


def round32(n):
    return (int(n) + KSUB - 1) // KSUB * KSUB


def device_arg(t, name, dtype, device, shape=None):
    """t checked before its raw pointer goes to a native call, returned
    contiguous: a torch tensor of dtype on device whose shape matches
    (None entries match any extent).  The native calls read and write as
    many elements as their size arguments say, so a host tensor, another
    dtype or a short array must stop here with a Python error, not become
    an out-of-bounds access in a kernel."""
    torch = _torch()
    if not isinstance(t, torch.Tensor):
        raise TypeError('%s: a torch tensor on %s expected, got %s'
                        % (name, device, type(t).__name__))
    if t.device != device:
        raise ValueError('%s is on %s, expected %s' % (name, t.device, device))
    if t.dtype != dtype:
        raise TypeError('%s is %s, expected %s' % (name, t.dtype, dtype))
    if shape is not None and (t.dim() != len(shape) or any(
            s is not None and int(a) != int(s) for a, s in zip(t.shape, shape))):
        raise ValueError('%s has shape %s, expected (%s)'
                         % (name, tuple(t.shape),
                            ', '.join('*' if s is None else str(int(s)) for s in shape)))
    return t.contiguous()


def device_out(t, name, dtype, device, shape):
    """An output buffer: as device_arg, and already contiguous (a copy
    would not receive the result)."""
    device_arg(t, name, dtype, device, shape)
    if not t.is_contiguous():
        raise ValueError('%s must be contiguous' % name)
    return t


F_ENGINES = {'library': 0, 'tc': 1}


def set_f_engine(name):
    """Engine of the F product of the Ozaki split (process-wide): 'library'
    (the default, cuBLAS bf16 level GEMMs) or 'tc' (this library's tcgen05
    tensor-core kernel with the level combination fused); both give
    bitwise the same F.  Returns the previous engine's name."""
    if name not in F_ENGINES:
        raise ValueError('F engine must be one of %s' % sorted(F_ENGINES))
    prev = get_f_engine()
    _native.check(_native.lib().wb_ozaki_set_f_engine(F_ENGINES[name]),
                  'wb_ozaki_set_f_engine')
    return prev


def get_f_engine():
    code = int(_native.lib().wb_ozaki_get_f_engine())
    return {v: k for k, v in F_ENGINES.items()}[code]


def as_molecule(mol):
    """A Molecule from a Molecule or a PySCF Mole."""
    if isinstance(mol, Molecule):
        return mol
    if hasattr(mol, '_bas') and hasattr(mol, '_libcint_ctr_coeff'):
        return Molecule.from_pyscf(mol)
    raise TypeError('expected a Molecule or a PySCF Mole, got %r' % type(mol))


class CosxEngine:
    """Native COSX kernels for one molecule on one CUDA device.

    origin: the molecule-centred frame of the kernels (default: mean of the
    atom coordinates, as the reference's GpuKBuilder, gpu/sgx_k.py:564).
    """

    def __init__(self, mol, origin=None, pair_cutoff=1e-14, device=None):
        torch = _torch()
        self.mol = as_molecule(mol)
        coords = self.mol.atom_coords()
        self.origin = (coords.mean(axis=0) if origin is None
                       else np.asarray(origin, dtype=np.float64))
        if device is None:
            device = torch.cuda.current_device()
        if not isinstance(device, int):
            device = torch.device(device).index or 0
        self.device = torch.device('cuda', device)
        self._packed = self.mol.packed()
        self._basis = _wb_basis(self._packed)
        self._origin_c = np.ascontiguousarray(self.origin, dtype=np.float64)
        lib = _native.lib()
        handle = _native.ctypes.c_void_p()
        with torch.cuda.device(self.device):
            _native.check(lib.wb_cosx_create(_native.ctypes.byref(self._basis),
                                             _native.ptr(self._origin_c),
                                             float(pair_cutoff),
                                             _native.ctypes.byref(handle)),
                          'wb_cosx_create')
        self._h = handle
        info = _native.WbCosxInfo()
        _native.check(lib.wb_cosx_get_info(self._h, _native.ctypes.byref(info)))
        self.nao = int(info.nao)
        self.npairs = int(info.npairs)
        self.nprim_pairs = int(info.nprim_pairs)
        self.class_pairs = [int(x) for x in info.class_pairs]
        self.class_prim_pairs = [int(x) for x in info.class_prim_pairs]
        self.nvshell = int(info.nbas)
        self._ws = None
        self.last_stats = {}

    # -- lifetime -----------------------------------------------------------
    def close(self):
        if getattr(self, '_h', None):
            _native.lib().wb_cosx_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:                       # noqa: BLE001
            pass

    # -- helpers ------------------------------------------------------------
    def pair_table(self):
        """(npairs, 8) int64: ia0, ib0, pp0, npp|diag<<16, class, ish, jsh,
        model flops per point."""
        lib = _native.lib()
        rows = np.zeros((max(self.npairs, 1), 8), dtype=np.int64)
        n = lib.wb_cosx_export_pairs(self._h, _native.ptr(rows), self.npairs)
        return rows[:n]

    def workspace_bytes(self, npts, tile_pts=0):
        return int(_native.lib().wb_cosx_workspace_bytes(self._h, int(npts),
                                                         int(tile_pts)))

    def workspace(self, nbytes):
        torch = _torch()
        if self._ws is None or self._ws.numel() < nbytes:
            self._ws = None
            self._ws = torch.empty(int(nbytes), dtype=torch.uint8,
                                   device=self.device)
        return self._ws

    def relative(self, coords):
        """Absolute FP64 coordinates (host or device) -> kernel frame, on
        this engine's device."""
        torch = _torch()
        c = torch.as_tensor(coords, dtype=torch.float64, device=self.device)
        o = torch.as_tensor(self.origin, dtype=torch.float64, device=self.device)
        return (c - o).contiguous()

    @staticmethod
    def _stream():
        return _native.ctypes.c_void_p(_torch().cuda.current_stream().cuda_stream)

    def _grid_args(self, coords_rel, weights):
        """(coords_rel (npts, 3), weights (npts,)) FP64 on this engine's
        device, checked and contiguous, and npts."""
        torch = _torch()
        c = device_arg(coords_rel, 'coords_rel', torch.float64, self.device, (None, 3))
        n = int(c.shape[0])
        w = device_arg(weights, 'weights', torch.float64, self.device, (n,))
        return c, w, n

    def _dm_arg(self, qd, name='qd'):
        return device_arg(qd, name, _torch().float64, self.device, (self.nao, self.nao))

    # -- entry points ---------------------------------------------------------
    def get_k(self, coords_rel, weights, qd, omega, tile_tol=1e-11,
              tile_pts=0, gemm='ozaki', out=None, stats=True,
              profile=False):
        """Unsymmetrised K = X^T (w o G) (nao, nao) FP64 on the device.
        coords_rel (npts, 3) FP64 device (kernel frame), weights (npts,) FP64
        device, qd (nao, nao) FP64 device = proj @ dm.  gemm: 'ozaki'
        (FP64-accurate split on the bf16 tensor cores, default), 'native'
        (cuBLAS DGEMM) or 'emulated' (cuBLAS FP64 emulation)."""
        torch = _torch()
        coords_rel, weights, npts = self._grid_args(coords_rel, weights)
        qd = self._dm_arg(qd)
        nbytes = self.workspace_bytes(npts, tile_pts)
        ws = self.workspace(nbytes)
        if out is None:
            out = torch.empty((self.nao, self.nao), dtype=torch.float64,
                              device=self.device)
        device_out(out, 'out', torch.float64, self.device, (self.nao, self.nao))
        st = _native.WbCosxStats() if stats else None
        flags = _native.GEMM_MODES[gemm]
        if profile and stats:
            flags |= _native.WB_K_PROFILE
        _native.check(_native.lib().wb_cosx_get_k(
            self._h, _native.ptr(coords_rel), _native.ptr(weights), npts,
            _native.ptr(qd), float(omega), float(tile_tol),
            int(tile_pts), flags, _native.ptr(out), _native.ptr(ws), nbytes,
            self._stream(), _native.ctypes.byref(st) if st is not None else None),
            'wb_cosx_get_k')
        if st is not None:
            self.last_stats = st.as_dict()
        return out

    def get_k_multi(self, coords_rel, weights, qd, omegas, tile_tol=1e-11,
                    tile_pts=0, gemm='ozaki', out=None, stats=True,
                    profile=False):
        """get_k for several omegas and one density in one call: the AO
        values, F and the block statistics of each tile serve every omega.
        Returns (len(omegas), nao, nao) FP64 on the device; out[j] is what
        get_k(..., omegas[j]) returns."""
        torch = _torch()
        om = [float(w) for w in omegas]
        if not om:
            raise ValueError('omegas is empty')
        coords_rel, weights, npts = self._grid_args(coords_rel, weights)
        qd = self._dm_arg(qd)
        nbytes = self.workspace_bytes(npts, tile_pts)
        ws = self.workspace(nbytes)
        if out is None:
            out = torch.empty((len(om), self.nao, self.nao), dtype=torch.float64,
                              device=self.device)
        device_out(out, 'out', torch.float64, self.device, (len(om), self.nao, self.nao))
        st = _native.WbCosxStats() if stats else None
        flags = _native.GEMM_MODES[gemm]
        if profile and stats:
            flags |= _native.WB_K_PROFILE
        arr = (_native.ctypes.c_double * len(om))(*om)
        _native.check(_native.lib().wb_cosx_get_k_multi(
            self._h, _native.ptr(coords_rel), _native.ptr(weights), npts,
            _native.ptr(qd), len(om), arr, float(tile_tol),
            int(tile_pts), flags, _native.ptr(out), _native.ptr(ws), nbytes,
            self._stream(), _native.ctypes.byref(st) if st is not None else None),
            'wb_cosx_get_k_multi')
        if st is not None:
            self.last_stats = st.as_dict()
        return out

    def k_grad(self, coords_rel, weights, dm, omega, tile_tol=0.0):
        """Nuclear gradient (natm, 3) FP64 (host) of E = -1/4 tr(D K(omega))
        at fixed D, grid points and weights (SGX with the grid response
        off), for the plain SGX K (dm the symmetric density, no projector);
        FP64 throughout (wb_cosx_k_grad)."""
        torch = _torch()
        coords_rel, weights, npts = self._grid_args(coords_rel, weights)
        natm = int(self.mol.natm)
        nbytes = int(_native.lib().wb_cosx_k_grad_workspace_bytes(self._h, npts, natm))
        ws = self.workspace(nbytes)
        out = torch.empty((natm, 3), dtype=torch.float64, device=self.device)
        d = self._dm_arg(torch.as_tensor(dm, dtype=torch.float64, device=self.device),
                         'dm')
        _native.check(_native.lib().wb_cosx_k_grad(
            self._h, _native.ptr(coords_rel), _native.ptr(weights), npts,
            _native.ptr(d), float(omega), float(tile_tol), natm, _native.ptr(out),
            _native.ptr(ws), nbytes, self._stream()), 'wb_cosx_k_grad')
        return out.cpu().numpy()

    def capture_k_multi(self, coords_rel, weights, omegas, tile_tol=1e-11,
                        gemm='ozaki'):
        """A get_k_multi build captured in a CUDA graph on fixed buffers:
        returns a KBuildGraph whose run(dm) copies dm into its density
        buffer, replays the graph and returns the symmetrised K
        (len(omegas), nao, nao) on the device (its own output buffer,
        overwritten by the next run).  coords_rel and weights must stay
        alive and unchanged.  One warm-up build runs first (it allocates
        the workspace and the block-order arrays, which a capture must
        not)."""
        return KBuildGraph(self, coords_rel, weights, omegas, tile_tol, gemm)

    def get_k_fp64(self, coords_rel, weights, qd, omegas, tile_tol=1e-11,
                   out=None, stats=True):
        """The plain FP64 form of get_k_multi: FP64 AO values, F = X QD kept
        in FP64 (cuBLAS DGEMM), the same screen, G from the FP64 class
        kernels (accumulated in FP64), K = X^T (w o G) by cuBLAS DGEMM; the
        whole grid is one tile.  Returns (len(omegas), nao, nao) FP64 on
        the device, unsymmetrised.  The first call on an engine uploads the
        FP64 pair tables (synchronous)."""
        torch = _torch()
        om = [float(w) for w in omegas]
        if not om:
            raise ValueError('omegas is empty')
        coords_rel, weights, npts = self._grid_args(coords_rel, weights)
        qd = self._dm_arg(qd)
        nbytes = int(_native.lib().wb_cosx_fp64_workspace_bytes(self._h, npts))
        ws = self.workspace(nbytes)
        if out is None:
            out = torch.empty((len(om), self.nao, self.nao), dtype=torch.float64,
                              device=self.device)
        device_out(out, 'out', torch.float64, self.device, (len(om), self.nao, self.nao))
        st = _native.WbCosxStats() if stats else None
        arr = (_native.ctypes.c_double * len(om))(*om)
        _native.check(_native.lib().wb_cosx_get_k_fp64(
            self._h, _native.ptr(coords_rel), _native.ptr(weights), npts,
            _native.ptr(qd), len(om), arr, float(tile_tol),
            _native.ptr(out), _native.ptr(ws), nbytes, self._stream(),
            _native.ctypes.byref(st) if st is not None else None),
            'wb_cosx_get_k_fp64')
        if st is not None:
            self.last_stats = st.as_dict()
        return out

    def g(self, coords_rel, weights, f, omega, tile_tol=0.0, out=None,
          stats=True):
        """G (nao, ld) FP32 from F (nao, ld) FP32 AO-major, one tile."""
        torch = _torch()
        coords_rel, weights, npts = self._grid_args(coords_rel, weights)
        ld = round32(npts)
        f = device_arg(f, 'f', torch.float32, self.device, (self.nao, ld))
        # the G-only call needs no X / F / G buffers in the workspace
        nbytes = self.workspace_bytes(npts)
        ws = self.workspace(nbytes)
        if out is None:
            out = torch.empty((self.nao, ld), dtype=torch.float32,
                              device=self.device)
        device_out(out, 'out', torch.float32, self.device, (self.nao, ld))
        st = _native.WbCosxStats() if stats else None
        _native.check(_native.lib().wb_cosx_g(
            self._h, _native.ptr(coords_rel), _native.ptr(weights), npts,
            _native.ptr(f), float(omega), float(tile_tol),
            _native.ptr(out), _native.ptr(ws), nbytes, self._stream(),
            _native.ctypes.byref(st) if st is not None else None), 'wb_cosx_g')
        if st is not None:
            self.last_stats = st.as_dict()
        return out

    def int1e(self, nuc_xyz=None, nuc_z=None):
        """(S, T, V) FP64 (nao, nao) on the device: overlap, kinetic energy
        and nuclear attraction (wb_scf_int1e).  The nuclei default to the
        molecule's own (absolute frame, bohr; all-electron charges)."""
        torch = _torch()
        xyz = np.ascontiguousarray(self.mol.atom_coords() if nuc_xyz is None
                                   else nuc_xyz, dtype=np.float64).reshape(-1, 3)
        z = np.ascontiguousarray(self.mol.atom_charges() if nuc_z is None else nuc_z,
                                 dtype=np.float64).ravel()
        if len(z) != len(xyz):
            raise ValueError('one charge per nucleus')
        out = [torch.empty((self.nao, self.nao), dtype=torch.float64, device=self.device)
               for _ in range(3)]
        _native.check(_native.lib().wb_scf_int1e(
            self._h, len(z), xyz.ctypes.data_as(_native.ctypes.c_void_p),
            z.ctypes.data_as(_native.ctypes.c_void_p), *[_native.ptr(o) for o in out],
            self._stream()), 'wb_scf_int1e')
        return tuple(out)

    def hartree(self, coords_rel, dm, tol=0.0, fp64=True, out=None, stats=False):
        """Hartree potential (npts,) FP64 on the device at coords_rel (the
        kernel frame) of the symmetric density dm (wb_hartree); tol screens
        (block, pair) tasks by the locked bound times the pair's |D|."""
        torch = _torch()
        coords_rel = device_arg(coords_rel, 'coords_rel', torch.float64, self.device)
        if coords_rel.dim() != 2 or coords_rel.shape[1] != 3:
            raise ValueError('coords_rel must be (npts, 3)')
        npts = int(coords_rel.shape[0])
        D = self._dm_arg(dm, 'dm')
        nbytes = int(_native.lib().wb_hartree_workspace_bytes(self._h, npts))
        ws = self.workspace(nbytes)
        if out is None:
            out = torch.empty(npts, dtype=torch.float64, device=self.device)
        device_out(out, 'out', torch.float64, self.device, (npts,))
        kept = _native.ctypes.c_int64(-1)
        _native.check(_native.lib().wb_hartree(
            self._h, _native.ptr(coords_rel), npts, _native.ptr(D), float(tol),
            1 if fp64 else 0, _native.ptr(out), _native.ptr(ws), nbytes,
            self._stream(), _native.ctypes.byref(kept) if stats else None),
            'wb_hartree')
        if stats:
            self.last_hartree_kept = int(kept.value)
        return out

    def screen_mask(self, coords_rel, weights, f, tile_tol, level=0):
        """(nblk, npairs) uint8 device mask of the tasks the fused G
        kernels keep at tile_tol, for blocks of 32 << level points; pair k
        is row k of pair_table() (wb_cosx_screen_mask)."""
        torch = _torch()
        if level not in (0, 1, 2):
            raise ValueError('level must be 0, 1 or 2')
        coords_rel, weights, npts = self._grid_args(coords_rel, weights)
        ld = round32(npts)
        f = device_arg(f, 'f', torch.float32, self.device, (self.nao, ld))
        nbytes = self.workspace_bytes(npts)
        ws = self.workspace(nbytes)
        nblk = -(-ld // (32 << level))
        keep = torch.zeros((nblk, max(self.npairs, 1)), dtype=torch.uint8,
                           device=self.device)
        _native.check(_native.lib().wb_cosx_screen_mask(
            self._h, _native.ptr(coords_rel), _native.ptr(weights), npts,
            _native.ptr(f), float(tile_tol), int(level), _native.ptr(keep),
            _native.ptr(ws), nbytes, self._stream()), 'wb_cosx_screen_mask')
        return keep[:, :self.npairs]

    def g_multi(self, coords_rel, weights, f, omegas, tile_tol=0.0, out=None,
                stats=True):
        """G for several omegas from one F: (len(omegas), nao, ld) FP32,
        out[j] equal to g(..., omegas[j]); omega pairs share one pass of
        the two-omega class kernels."""
        torch = _torch()
        om = [float(w) for w in omegas]
        if not om:
            raise ValueError('omegas is empty')
        coords_rel, weights, npts = self._grid_args(coords_rel, weights)
        ld = round32(npts)
        f = device_arg(f, 'f', torch.float32, self.device, (self.nao, ld))
        nbytes = self.workspace_bytes(npts)
        ws = self.workspace(nbytes)
        if out is None:
            out = torch.empty((len(om), self.nao, ld), dtype=torch.float32,
                              device=self.device)
        device_out(out, 'out', torch.float32, self.device, (len(om), self.nao, ld))
        st = _native.WbCosxStats() if stats else None
        arr = (_native.ctypes.c_double * len(om))(*om)
        _native.check(_native.lib().wb_cosx_g_multi(
            self._h, _native.ptr(coords_rel), _native.ptr(weights), npts,
            _native.ptr(f), len(om), arr, float(tile_tol),
            _native.ptr(out), _native.ptr(ws), nbytes, self._stream(),
            _native.ctypes.byref(st) if st is not None else None),
            'wb_cosx_g_multi')
        if st is not None:
            self.last_stats = st.as_dict()
        return out

    def ozaki_f(self, X, qd, fp64=False):
        """F (nao, ld) = X^T-side product QD^T X through the bf16 Ozaki split:
        FP32 (fl32 of the product) or, with fp64, FP64 (the 42-bit level
        sums rounded once)."""
        torch = _torch()
        X = device_arg(X, 'X', torch.float64, self.device, (self.nao, None))
        qd = self._dm_arg(qd)
        ld = int(X.shape[1])
        nbytes = int(_native.lib().wb_ozaki_workspace_bytes(self.nao, ld))
        ws = self.workspace(nbytes)
        dt = torch.float64 if fp64 else torch.float32
        out = torch.empty((self.nao, ld), dtype=dt, device=self.device)
        fn = 'wb_cosx_ozaki_f64' if fp64 else 'wb_cosx_ozaki_f'
        _native.check(getattr(_native.lib(), fn)(
            self._h, _native.ptr(X), _native.ptr(qd), ld,
            _native.ptr(out), _native.ptr(ws), nbytes, self._stream()), fn)
        return out

    def ozaki_k(self, X, G, weights, out=None, accumulate=False):
        """K (nao, nao) FP64 = X^T (w o G) through the bf16 Ozaki split; G
        FP32, or FP64 (w o G then formed from the FP64 values)."""
        torch = _torch()
        X = device_arg(X, 'X', torch.float64, self.device, (self.nao, None))
        ld = int(X.shape[1])
        g64 = getattr(G, 'dtype', None) == torch.float64
        G = device_arg(G, 'G', torch.float64 if g64 else torch.float32, self.device,
                       (self.nao, ld))
        weights = device_arg(weights, 'weights', torch.float64, self.device, (None,))
        npts = int(weights.shape[0])
        if npts > ld:
            raise ValueError('%d weights for %d columns of X' % (npts, ld))
        nbytes = int(_native.lib().wb_ozaki_workspace_bytes(self.nao, ld))
        ws = self.workspace(nbytes)
        if out is None:
            out = torch.zeros((self.nao, self.nao), dtype=torch.float64,
                              device=self.device)
        device_out(out, 'out', torch.float64, self.device, (self.nao, self.nao))
        fn = 'wb_cosx_ozaki_k64' if g64 else 'wb_cosx_ozaki_k'
        _native.check(getattr(_native.lib(), fn)(
            self._h, _native.ptr(X), _native.ptr(G), _native.ptr(weights), npts,
            1 if accumulate else 0, _native.ptr(out), _native.ptr(ws), nbytes,
            self._stream()), fn)
        return out

    def ao_eval(self, coords_rel, out=None):
        """X (nao, ld) FP64 AO-major."""
        torch = _torch()
        coords_rel = device_arg(coords_rel, 'coords_rel', torch.float64, self.device,
                                (None, 3))
        npts = int(coords_rel.shape[0])
        if out is None:
            out = torch.empty((self.nao, round32(npts)), dtype=torch.float64,
                              device=self.device)
        device_out(out, 'out', torch.float64, self.device, (self.nao, round32(npts)))
        _native.check(_native.lib().wb_ao_eval(
            self._h, _native.ptr(coords_rel), npts, _native.ptr(out),
            self._stream()), 'wb_ao_eval')
        return out

    def ao_eval_deriv1(self, coords_rel, out=None):
        """X and its gradients (4, nao, ld) FP64 AO-major."""
        torch = _torch()
        coords_rel = device_arg(coords_rel, 'coords_rel', torch.float64, self.device,
                                (None, 3))
        npts = int(coords_rel.shape[0])
        if out is None:
            out = torch.empty((4, self.nao, round32(npts)), dtype=torch.float64,
                              device=self.device)
        device_out(out, 'out', torch.float64, self.device, (4, self.nao, round32(npts)))
        _native.check(_native.lib().wb_ao_eval_deriv1(
            self._h, _native.ptr(coords_rel), npts, _native.ptr(out),
            self._stream()), 'wb_ao_eval_deriv1')
        return out

    def xc_rho(self, X, T, npts, mgga):
        """Semilocal XC density parameters (5, ld) FP64 (rho, grad, tau) from
        X (4, nao, ld) FP64 and T (1 or 4, nao, ld) FP32 = fl32(dm^T X_d)."""
        torch = _torch()
        X = device_arg(X, 'X', torch.float64, self.device, (4, self.nao, None))
        ld = int(X.shape[2])
        T = device_arg(T, 'T', torch.float32, self.device, (None, self.nao, ld))
        if T.shape[0] < (4 if mgga else 1) or not 0 <= int(npts) <= ld:
            raise ValueError('T needs %d planes and npts <= %d'
                             % (4 if mgga else 1, ld))
        out = torch.empty((5, ld), dtype=torch.float64, device=self.device)
        _native.check(_native.lib().wb_xc_rho(
            self._h, _native.ptr(X), _native.ptr(T), int(npts), ld,
            1 if mgga else 0, _native.ptr(out), self._stream()), 'wb_xc_rho')
        return out

    def xc_aow(self, X, v, npts, mgga):
        """Fock-side planes (1 or 4, nao, ld) FP32 from X and the
        density-parameter derivatives v (5, ld) FP64."""
        torch = _torch()
        X = device_arg(X, 'X', torch.float64, self.device, (4, self.nao, None))
        ld = int(X.shape[2])
        v = device_arg(v, 'v', torch.float64, self.device, (5, ld))
        if not 0 <= int(npts) <= ld:
            raise ValueError('npts must be in [0, %d]' % ld)
        out = torch.empty((4 if mgga else 1, self.nao, ld), dtype=torch.float32,
                          device=self.device)
        _native.check(_native.lib().wb_xc_aow(
            self._h, _native.ptr(X), _native.ptr(v), int(npts), ld,
            1 if mgga else 0, _native.ptr(out), self._stream()), 'wb_xc_aow')
        return out

    def int3c1e_dense(self, coords_rel, omega=0.0):
        """Dense (npts, nao, nao) FP32 contracted spherical integrals
        (validation only; refuses more than 2 GiB)."""
        torch = _torch()
        coords_rel = device_arg(coords_rel, 'coords_rel', torch.float64, self.device,
                                (None, 3))
        npts = int(coords_rel.shape[0])
        need = npts * self.nao * self.nao * 4
        if need > (2 << 30):
            raise MemoryError('dense int3c1e needs %d bytes' % need)
        out = torch.empty((npts, self.nao, self.nao), dtype=torch.float32,
                          device=self.device)
        _native.check(_native.lib().wb_int3c1e_dense(
            self._h, _native.ptr(coords_rel), npts, float(omega),
            _native.ptr(out), self._stream()), 'wb_int3c1e_dense')
        return out


class KBuildGraph:
    """One multi-omega K build of an engine captured in a CUDA graph (see
    CosxEngine.capture_k_multi).  Every launch of the build (AO values,
    the F split, block statistics, the class kernels on the engine's class
    streams, the class-buffer sums, the K split) and the symmetrisation
    replay with one graph launch; the block order of each replay is the
    one the previous replay's kernels recorded on the device.  Not
    thread-safe: one run at a time per graph (and per engine)."""

    def __init__(self, eng, coords_rel, weights, omegas, tile_tol, gemm):
        torch = _torch()
        self.eng = eng
        self.omegas = tuple(float(w) for w in omegas)
        self._coords, self._weights = coords_rel, weights
        self.qd = torch.zeros((eng.nao, eng.nao), dtype=torch.float64,
                              device=eng.device)
        self._k = torch.empty((len(self.omegas), eng.nao, eng.nao),
                              dtype=torch.float64, device=eng.device)
        args = dict(tile_tol=tile_tol, gemm=gemm, out=self._k, stats=False)
        side = torch.cuda.Stream(device=eng.device)
        side.wait_stream(torch.cuda.current_stream(eng.device))
        with torch.cuda.stream(side):
            # warm-up: workspace, block-order arrays, cuBLAS kernel choice
            eng.get_k_multi(coords_rel, weights, self.qd, self.omegas, **args)
        torch.cuda.current_stream(eng.device).wait_stream(side)
        side.synchronize()
        self.graph = torch.cuda.CUDAGraph()
        with torch.cuda.graph(self.graph, capture_error_mode='thread_local'):
            eng.get_k_multi(coords_rel, weights, self.qd, self.omegas, **args)
            self.out = (self._k + self._k.transpose(1, 2)) * 0.5

    def run(self, dm):
        """dm (nao, nao) FP64, host or device -> symmetrised K on the device
        (this graph's output buffer)."""
        torch = _torch()
        dm = torch.as_tensor(dm, dtype=torch.float64)
        if tuple(dm.shape) != tuple(self.qd.shape):
            raise ValueError('dm has shape %s, expected %s'
                             % (tuple(dm.shape), tuple(self.qd.shape)))
        self.qd.copy_(dm, non_blocking=True)
        self.graph.replay()
        return self.out


def batch_workspace_bytes(engines, npts):
    """Per-molecule workspace bytes of a CosxBatch and the bytes of its
    shared scratch."""
    lib = _native.lib()
    ws, scr = [], 0
    for e, n in zip(engines, npts):
        s = _native.ctypes.c_size_t(0)
        ws.append(int(lib.wb_cosx_batch_workspace_bytes(e._h, int(n),
                                                        _native.ctypes.byref(s))))
        scr = max(scr, int(s.value))
    return ws, scr


class CosxBatch:
    """K builds of several molecules per call (wb_cosx_batch_*): one launch
    per class kernel over all molecules.  engines: one CosxEngine per
    molecule (each used only by this batch while it lives; its workspace
    is sized for its grid); grids: (coords_rel, weights) device tensors per
    molecule, kept alive and unchanged.  The AO values, grid coordinates
    and omega records are formed once here; run(qds) builds every K."""

    def __init__(self, engines, grids, omegas=(0.0, 0.3), tile_tol=1e-11,
                 gemm='ozaki'):
        torch = _torch()
        if not engines or len(engines) != len(grids):
            raise ValueError('one (coords_rel, weights) per engine')
        self.engines = list(engines)
        self.omegas = tuple(float(w) for w in omegas)
        if len(self.omegas) not in (1, 2):
            raise ValueError('1 or 2 omegas')
        self._grids = [e._grid_args(c, w)[:2] for e, (c, w) in zip(self.engines, grids)]
        n = len(self.engines)
        dev = self.engines[0].device
        P = _native.ctypes.c_void_p
        npts = [int(c.shape[0]) for c, _ in self._grids]
        wsb, scr = batch_workspace_bytes(self.engines, npts)
        ws = [e.workspace(b) for e, b in zip(self.engines, wsb)]
        self._scratch = torch.empty(max(scr, 1), dtype=torch.uint8, device=dev)
        self._hold = ws
        handles = (P * n)(*[e._h.value for e in self.engines])
        coords = (P * n)(*[c.data_ptr() for c, _ in self._grids])
        weights = (P * n)(*[w.data_ptr() for _, w in self._grids])
        npts_a = (_native.ctypes.c_int64 * n)(*npts)
        ws_a = (P * n)(*[t.data_ptr() for t in ws])
        wsb_a = (_native.ctypes.c_size_t * n)(*wsb)
        om = (_native.ctypes.c_double * len(self.omegas))(*self.omegas)
        out = P()
        with torch.cuda.device(dev):
            _native.check(_native.lib().wb_cosx_batch_create(
                n, handles, coords, weights, npts_a, ws_a, wsb_a,
                self._scratch.data_ptr(), self._scratch.numel(), len(self.omegas),
                om, float(tile_tol), _native.GEMM_MODES[gemm],
                CosxEngine._stream(), _native.ctypes.byref(out)),
                'wb_cosx_batch_create')
        self._b = out
        self.device = dev
        self.last_stats = {}

    def run(self, qds, out=None, stats=False):
        """qds: one (nao, nao) FP64 device tensor per molecule -> a list of
        (len(omegas), nao, nao) unsymmetrised K (out: the same, to reuse).
        A None density leaves its molecule out of the run (its entry of the
        result is None)."""
        torch = _torch()
        n = len(self.engines)
        if len(qds) != n:
            raise ValueError('one density per molecule')
        if all(q is None for q in qds):
            raise ValueError('at least one density')
        if out is None:
            out = [None if q is None else
                   torch.empty((len(self.omegas), e.nao, e.nao), dtype=torch.float64,
                               device=self.device) for q, e in zip(qds, self.engines)]
        P = _native.ctypes.c_void_p
        qd_c = [None if q is None else e._dm_arg(q) for q, e in zip(qds, self.engines)]
        if len(out) != n:
            raise ValueError('one output per molecule')
        for q, k, e in zip(qd_c, out, self.engines):
            if q is not None:
                device_out(k, 'out', torch.float64, e.device,
                           (len(self.omegas), e.nao, e.nao))
        st = _native.WbCosxStats() if stats else None
        _native.check(_native.lib().wb_cosx_batch_run(
            self._b, (P * n)(*[None if q is None else q.data_ptr() for q in qd_c]),
            (P * n)(*[None if q is None else k.data_ptr() for q, k in zip(qd_c, out)]),
            CosxEngine._stream(), _native.ctypes.byref(st) if st is not None else None),
            'wb_cosx_batch_run')
        if st is not None:
            self.last_stats = st.as_dict()
        return [None if q is None else k for q, k in zip(qd_c, out)]

    def close(self):
        if getattr(self, '_b', None):
            _native.lib().wb_cosx_batch_destroy(self._b)
            self._b = None

    def __del__(self):
        try:
            self.close()
        except Exception:                       # noqa: BLE001
            pass


def _wb_basis(p):
    """The C-ABI basis view of Molecule.packed() p (p must outlive it)."""
    return _native.WbBasis(
        p['natm'], p['nbas'], _native.ptr(p['atom_coords']),
        _native.ptr(p['shell_atom']), _native.ptr(p['shell_l']),
        _native.ptr(p['shell_nprim']), _native.ptr(p['shell_nctr']),
        _native.ptr(p['shell_exp_off']), _native.ptr(p['shell_coef_off']),
        _native.ptr(p['exps']), _native.ptr(p['coeffs']))


def model_flops_per_point(mol, pair_cutoff=1e-14):
    """(model flops per grid point over the kept shell pairs, number of
    pairs) -- the work of one point with no task screening, on the host."""
    p = as_molecule(mol).packed()
    b = _wb_basis(p)
    out = _native.ctypes.c_double()
    n = _native.ctypes.c_int64()
    _native.check(_native.lib().wb_model_flops_per_point(
        _native.ctypes.byref(b), float(pair_cutoff), _native.ctypes.byref(out),
        _native.ctypes.byref(n)), 'wb_model_flops_per_point')
    return float(out.value), int(n.value)


def boys_eval(T, nmax):
    """FP32 Boys F_0..F_nmax of a CUDA float32 tensor: (nmax+1, n)."""
    torch = _torch()
    if not 0 <= nmax <= 6:
        raise ValueError('nmax must be 0..6')
    T = T.to(torch.float32).contiguous()
    out = torch.empty((nmax + 1, T.numel()), dtype=torch.float32, device=T.device)
    _native.check(_native.lib().wb_boys_fp32(
        _native.ptr(T), T.numel(), int(nmax), _native.ptr(out),
        CosxEngine._stream()), 'wb_boys_fp32')
    return out


def boys_f64_host(nmax, t):
    """FP64 Boys F_0..F_nmax at one argument (the library's host routine)."""
    out = np.zeros(nmax + 1)
    _native.check(_native.lib().wb_boys_f64_host(int(nmax), float(t),
                                                 _native.ptr(out)))
    return out


def becke_partition(points, owner, atom_coords):
    """Becke fuzzy-cell weight of each point's owner atom (host, native)."""
    points = np.ascontiguousarray(points, dtype=np.float64)
    owner = np.ascontiguousarray(owner, dtype=np.int32)
    atoms = np.ascontiguousarray(atom_coords, dtype=np.float64)
    out = np.zeros(len(points))
    _native.check(_native.lib().wb_becke_partition(
        _native.ptr(points), len(points), _native.ptr(owner), _native.ptr(atoms),
        len(atoms), _native.ptr(out)), 'wb_becke_partition')
    return out
