"""Runs the reference's own CUDA kernels on this GPU (the GPU-side baseline
of bench.py).  TEST INFRASTRUCTURE ONLY.

``RefGpu(tag)`` loads oracle/_ref/libref_gpu.so and the reference's packed
pair data (oracle/_ref/ref_pairs_<tag>.npz) onto the device.
``g_phase(coords, weights, F, omega)`` runs the reference's G phase of one
K build exactly as GpuKBuilder.get_k does (gpu/sgx_k.py:717-735, 754-781,
866-924): per grid tile of (SMs x 32 warps x 32) points the sub-block shell
maxima (|F| w through the shell-indicator SGEMM, max over 32 points), the
centroid / radius per sub-block (FP64, the radius rounded up), the
screening kernel sgx_screen_mask, the per-class CSR task lists (row-major
nonzero, counts, prefix sum) and one sgx_k_cls<LA,LB> launch per non-empty
class (sgx_k_tile for generally contracted pairs), in class order.  The
screen and the class launches are timed with CUDA events on the stream;
the CSR build (a host round trip per class in the reference too) is timed
apart.  ``vv10(xyz, q, w0, kappa)`` runs vv10_kernel_sum over 65,536-point
launch chunks.
"""
import ctypes
import os

import numpy as np

import oracle

KSUB = 32
WARPS_MAX = 4
WARPS_PER_SM = 32
GENERIC = 16
SAFETY = 1.001


def available(tag='water27_svp'):
    """None when the arm can run, else the reason (one line)."""
    if not os.path.exists(os.path.join(oracle.REF_DIR, 'ref_kernels.cuh')):
        return 'reference kernels not extracted (oracle/_ref/ref_kernels.cuh missing)'
    if not os.path.exists(os.path.join(oracle.REF_DIR, 'ref_pairs_%s.npz' % tag)):
        return 'reference pair data for %s missing' % tag
    return None


class _Pairs(ctypes.Structure):
    _fields_ = [(n, ctypes.c_void_p) for n in (
        'sh_dims', 'sh_Mc', 'sh_MT', 'sh_Mc_lo', 'sh_MT_lo', 'pair_sh', 'prim_p',
        'prim_prefac', 'prim_prefac_lo', 'prim_P_hi', 'prim_P_lo', 'prim_E')]


def _p(t):
    return ctypes.c_void_p(t.data_ptr())


class RefGpu:
    def __init__(self, tag='water27_svp', device=0):
        import torch
        lib_path = oracle.build_ref_gpu()
        if lib_path is None:
            raise RuntimeError(available(tag))
        self.lib = ctypes.CDLL(lib_path)
        self.lib.ref_max_threads.argtypes = [ctypes.c_int]
        I, P, D = ctypes.c_int, ctypes.c_void_p, ctypes.c_double
        self.lib.ref_cls_launch.argtypes = [I, P] + [P] * 9 + [I] * 4 + [D, P, I, P]
        self.lib.ref_screen_launch.argtypes = [P] * 10 + [I, I, I, ctypes.c_float, P, P]
        self.lib.ref_vv10_launch.argtypes = [P] * 4 + [I] + [P] * 4
        self.dev = torch.device('cuda', device)
        d = np.load(os.path.join(oracle.REF_DIR, 'ref_pairs_%s.npz' % tag))
        self.t = {k: torch.as_tensor(np.ascontiguousarray(d[k]), device=self.dev)
                  for k in d.files if d[k].ndim > 0}
        self.nao = int(d['nao'])
        self.npairs = int(d['npairs'])
        self.origin = np.asarray(d['origin'], dtype=np.float64)
        self.pairs = _Pairs(*[_p(self.t[n]) for n, _ in _Pairs._fields_])
        ao_loc = d['ao_loc']
        nbas = len(ao_loc) - 1
        ind = torch.zeros((self.nao, nbas), dtype=torch.float32, device=self.dev)
        for s in range(nbas):
            ind[ao_loc[s]:ao_loc[s + 1], s] = 1.0
        self.shell_ind = ind
        self.nbas = nbas
        cls = self.t['pair_class']
        self.class_pairs = [torch.nonzero(cls == c).flatten().to(torch.int32)
                            for c in range(GENERIC + 1)]
        self.warps = [max(1, min(WARPS_MAX, self.lib.ref_max_threads(c) // 32))
                      for c in range(GENERIC + 1)]
        self.nsm = torch.cuda.get_device_properties(self.dev).multi_processor_count

    def tile_points(self):
        """The reference's automatic tile: SMs x 32 warps x 32 points
        (GpuKBuilder._auto_blksize, memory never binds on this GPU)."""
        return self.nsm * WARPS_PER_SM * KSUB

    def g_phase(self, coords, weights, F, omega, tile_tol=1e-11):
        """coords (npts, 3) FP64 host (absolute frame), weights (npts,) FP64
        host, F (npts, nao) FP32 device, point-major.  Returns (G (npts,
        nao) FP32 device, stats dict)."""
        import torch
        stream = torch.cuda.current_stream(self.dev)
        sp = ctypes.c_void_p(stream.cuda_stream)
        npts = len(weights)
        c64 = np.asarray(coords, dtype=np.float64) - self.origin
        c32 = c64.astype(np.float32)
        c32lo = (c64 - c32.astype(np.float64)).astype(np.float32)
        cd = torch.as_tensor(c32, device=self.dev)
        cdl = torch.as_tensor(c32lo, device=self.dev)
        c64d = torch.as_tensor(c64, device=self.dev)
        w64 = torch.as_tensor(np.asarray(weights, dtype=np.float64), device=self.dev)
        key = 'w%g_' % omega
        tp_hi, tp_lo, cn_hi, cn_lo = (self.t[key + n] for n in ('tp_hi', 'tp_lo',
                                                                'cn_hi', 'cn_lo'))
        G = torch.zeros((npts, self.nao), dtype=torch.float32, device=self.dev)
        tile = self.tile_points()
        ev = lambda: torch.cuda.Event(enable_timing=True)
        t_screen = t_cls = t_csr = 0.0
        kept = 0
        for i0 in range(0, npts, tile):
            i1 = min(npts, i0 + tile)
            n = i1 - i0
            nsub = -(-n // KSUB)
            e0, e1, e2, e3 = ev(), ev(), ev(), ev()
            e0.record(stream)
            Ft = F[i0:i1]
            fw = Ft.abs() * w64[i0:i1].to(torch.float32)[:, None]
            seg = fw @ self.shell_ind
            pad = nsub * KSUB - n
            c = c64d[i0:i1]
            valid = torch.ones(n, dtype=torch.float64, device=self.dev)
            if pad:
                seg = torch.cat([seg, torch.zeros((pad, self.nbas), dtype=seg.dtype,
                                                  device=self.dev)])
                c = torch.cat([c, torch.zeros((pad, 3), dtype=c.dtype, device=self.dev)])
                valid = torch.cat([valid, torch.zeros(pad, dtype=valid.dtype,
                                                      device=self.dev)])
            msh = seg.reshape(nsub, KSUB, -1).amax(dim=1).contiguous()
            c = c.reshape(nsub, KSUB, 3)
            valid = valid.reshape(nsub, KSUB)
            cen = (c * valid[:, :, None]).sum(dim=1) / valid.sum(dim=1)[:, None]
            rad = (torch.sqrt(((c - cen[:, None, :]) ** 2).sum(dim=2)) * valid).amax(dim=1)
            cen32 = cen.to(torch.float32).contiguous()
            rad32 = torch.nextafter(rad.to(torch.float32),
                                    torch.tensor(float('inf'), device=self.dev))
            keep = torch.empty((nsub, self.npairs), dtype=torch.uint8, device=self.dev)
            st = self.lib.ref_screen_launch(
                _p(cen32), _p(rad32), _p(msh), _p(self.t['scr_P']), _p(self.t['scr_pref']),
                _p(self.t['scr_pp']), _p(self.t['scr_poff']), _p(self.t['scr_tau']),
                _p(self.t['scr_ish']), _p(self.t['scr_jsh']), nsub, self.npairs,
                self.nbas, float(tile_tol / SAFETY), _p(keep), sp)
            if st:
                raise RuntimeError('sgx_screen_mask launch: %d' % st)
            e1.record(stream)
            e1.synchronize()
            t_screen += e0.elapsed_time(e1)
            # per-class CSR (row-major nonzero: sub-block order, pair ids
            # ascending; deterministic), as _tasks_device builds it
            import time
            h0 = time.perf_counter()
            tasks = []
            for cls in range(GENERIC + 1):
                cols = self.class_pairs[cls]
                if cols.numel() == 0:
                    continue
                rows, cidx = torch.nonzero(keep[:, cols.long()], as_tuple=True)
                if rows.numel() == 0:
                    continue
                cnt = torch.bincount(rows, minlength=nsub)
                offs = torch.zeros(nsub + 1, dtype=torch.int32, device=self.dev)
                offs[1:] = torch.cumsum(cnt, 0).to(torch.int32)
                ids = cols[cidx].to(torch.int32).contiguous()
                kept += int(rows.numel())
                tasks.append((cls, offs, ids))
            torch.cuda.synchronize(self.dev)
            t_csr += time.perf_counter() - h0
            Gt = G[i0:i1]
            e2.record(stream)
            for cls, offs, ids in tasks:
                st = self.lib.ref_cls_launch(
                    cls, ctypes.byref(self.pairs), _p(tp_hi), _p(tp_lo), _p(cn_hi),
                    _p(cn_lo), _p(cd[i0:i1]), _p(cdl[i0:i1]), _p(Ft), _p(offs), _p(ids),
                    n, self.nao, KSUB, nsub, float(omega), _p(Gt), self.warps[cls], sp)
                if st:
                    raise RuntimeError('sgx_k class %d launch: %d' % (cls, st))
            e3.record(stream)
            e3.synchronize()
            t_cls += e2.elapsed_time(e3)
        return G, dict(screen_ms=t_screen, class_kernels_ms=t_cls,
                       csr_host_ms=t_csr * 1e3, tasks_kept=kept,
                       tasks_total=(-(-npts // KSUB)) * self.npairs,
                       tile_points=tile, warps_per_block=dict(enumerate(self.warps)))

    def vv10(self, xyz, q, w0, kappa):
        """F (raw sum, the reference applies -1.5 afterwards), U, W FP64 of
        the reference's fused kernel; inputs FP32 device."""
        import torch
        n = int(xyz.shape[0])
        out = [torch.zeros(n, dtype=torch.float64, device=self.dev) for _ in range(3)]
        sp = ctypes.c_void_p(torch.cuda.current_stream(self.dev).cuda_stream)
        st = self.lib.ref_vv10_launch(_p(xyz), _p(q), _p(w0), _p(kappa), n,
                                      *[_p(o) for o in out], sp)
        if st:
            raise RuntimeError('vv10_kernel_sum launch: %d' % st)
        return out
