"""Semilocal XC on the GPU: the NumInt.nr_rks replacement (reference:
pyscf_wb97mv_fast/gpu/xc.py:1-201).

``gpu_nr_rks(ctx, ni, mol, grids, xc_code, dms, ...) -> (nelec, excsum,
vmat)`` has NumInt.nr_rks's signature and result for one RKS density and an
LDA / GGA / MGGA (no laplacian) functional -- the wB97M-V case.  Per tile of
grid points (the whole grid when it fits):

    X      = AO values and gradients (4, nao, ld) FP64      wb_ao_eval_deriv1
    T_d    = fl32(dm^T X_d)  (d = 0, and x, y, z for MGGA)   wb_cosx_ozaki_f
    rho    = (rho, grad rho, tau) (5, ld) FP64               wb_xc_rho
    exc, v = functional on the host (FP64) + chain rule
    G      = 1/2 v0 X0 + sum_d v_d X_d  (+ 1/2 vtau X_d)     wb_xc_aow
    vmat  += X0^T (w o G0)  (+ sum_d X_d^T (w o G_d))        wb_cosx_ozaki_k

then vmat + vmat^T (+ the tau part once), nelec and excsum summed in FP64.
The two GEMMs are the FP64-accurate bf16 splits of the K build, rounded
once to FP32 where the reference's flow is FP32 (T and G), so the flow is at
least as accurate as the reference's FP32 path.

The functional is ``XcFunctional.eval(rho (5, P)) -> (exc, vrho, vsigma,
vtau)`` in the libxc convention (untransformed); ``PyscfLibxcFunctional``
is PySCF's own libxc (CPU FP64), the default.  ``chain_rule`` turns it into
density-parameter derivatives (transform_vxc for spin = 0).

Deliberate contract change, as for the K and VV10 hooks: no CPU fallback --
an unsupported case raises ``Unsupported``.  Importing this module does not
import PySCF or torch.
"""
import numpy as np

from pyscf_wb97mv_fast_gb300 import _native
from pyscf_wb97mv_fast_gb300.cosx import CosxEngine, as_molecule

SUPPORTED_XCTYPE = ('LDA', 'GGA', 'MGGA')
Unsupported = _native.Unsupported
# points per tile: X, T and G take (32 + 16 + 16) bytes per point and AO
DEFAULT_TILE_PTS = 1 << 20


def _torch():
    import torch
    return torch


class PyscfLibxcFunctional:
    """PySCF's libxc (CPU FP64) behind the XcFunctional interface
    (reference gpu/xc.py:36-49)."""

    def __init__(self, xc_code, ni):
        self.xc_code = xc_code
        self.ni = ni

    def eval(self, rho):
        """rho (5, P) = (rho, grad x, y, z, tau), host FP64."""
        exc, vxc = self.ni.eval_xc(self.xc_code, rho, spin=0, deriv=1)[:2]
        vsigma = vxc[1] if len(vxc) > 1 else None
        vtau = vxc[3] if len(vxc) > 3 else None
        return exc, vxc[0], vsigma, vtau


def chain_rule(rho, exc, vrho, vsigma, vtau):
    """libxc derivatives -> density-parameter derivatives (reference
    gpu/xc.py:96-116): v (5, P) = (vrho, 2 vsigma grad rho, vtau), zero rows
    where vsigma / vtau are absent.  Host FP64; returns (exc, v)."""
    rho = np.asarray(rho, dtype=np.float64)
    v = np.zeros((5, rho.shape[1]))
    v[0] = vrho
    if vsigma is not None:
        v[1:4] = 2.0 * np.asarray(vsigma, dtype=np.float64)[None] * rho[1:4]
    if vtau is not None:
        v[4] = vtau
    return np.asarray(exc, dtype=np.float64), v


class XcContext:
    """Per-mf state of the semilocal flow: the native engine (AO tables,
    the GEMM splits) and the functional factory."""

    def __init__(self, mol, functional_factory=None, tile_pts=DEFAULT_TILE_PTS,
                 device=None):
        self.mol = mol
        self.functional_factory = functional_factory
        self.tile_pts = int(tile_pts)
        self.device = device
        self.engine = None
        self.last_timings = None

    def build(self):
        if self.engine is None:
            self.engine = CosxEngine(as_molecule(self.mol), device=self.device)
        return self.engine

    def functional(self, xc_code, ni):
        if self.functional_factory is not None:
            return self.functional_factory(xc_code, ni)
        return PyscfLibxcFunctional(xc_code, ni)


def _prepare_dm(dms, hermi):
    dm = np.asarray(dms, dtype=np.float64)
    if dm.ndim == 3 and dm.shape[0] == 1:
        dm = dm[0]
    if dm.ndim != 2 or dm.shape[0] != dm.shape[1]:
        raise Unsupported(_native.WB_ERR_UNSUPPORTED,
                          'GPU XC path supports a single RKS density matrix')
    if hermi != 1:
        dm = 0.5 * (dm + dm.T)
    return np.ascontiguousarray(dm)


def _t_planes(eng, X, D, planes):
    """T_d = fl32(D^T X_d) (planes, nao, ld): the FP64-accurate split GEMM,
    or a cuBLAS DGEMM where nao is beyond one exact level sum."""
    torch = _torch()
    nao, ld = int(X.shape[1]), int(X.shape[2])
    T = torch.empty((planes, nao, ld), dtype=torch.float32, device=X.device)
    exact = 7 * nao < (1 << 14)
    for d in range(planes):
        if exact:
            T[d] = eng.ozaki_f(X[d], D)
        else:
            T[d] = (D.T @ X[d]).to(torch.float32)
    return T


def gpu_nr_rks(ctx, ni, mol, grids, xc_code, dms, relativity=0, hermi=1,
               max_memory=2000, verbose=None):
    """GPU replacement of NumInt.nr_rks (RKS ground state, one density)."""
    torch = _torch()
    xctype = ni._xc_type(xc_code)
    if xctype not in SUPPORTED_XCTYPE:
        raise Unsupported(_native.WB_ERR_UNSUPPORTED,
                          'xctype %r not supported on the GPU path' % (xctype,))
    if relativity not in (0, None):
        raise Unsupported(_native.WB_ERR_UNSUPPORTED,
                          'relativistic XC not supported')
    dm = _prepare_dm(dms, hermi)
    functional = ctx.functional(xc_code, ni)
    eng = ctx.build()
    if dm.shape[0] != eng.nao:
        raise Unsupported(_native.WB_ERR_INVALID_ARGUMENT,
                          'density matrix is %dx%d, the basis has %d AOs'
                          % (dm.shape[0], dm.shape[1], eng.nao))
    dev = eng.device
    mgga = xctype == 'MGGA'
    planes = 4 if mgga else 1
    D = torch.as_tensor(dm, device=dev)
    coords = np.asarray(grids.coords, dtype=np.float64)
    weights = np.asarray(grids.weights, dtype=np.float64)
    n = len(weights)
    vmat = torch.zeros((eng.nao, eng.nao), dtype=torch.float64, device=dev)
    vtau = torch.zeros_like(vmat) if mgga else None
    nelec = 0.0
    excsum = 0.0
    tile = max(32, ctx.tile_pts)
    for i0 in range(0, n, tile):
        i1 = min(n, i0 + tile)
        nt = i1 - i0
        c = eng.relative(coords[i0:i1])
        w = torch.as_tensor(weights[i0:i1], device=dev)
        X = eng.ao_eval_deriv1(c)                       # (4, nao, ld)
        T = _t_planes(eng, X, D, planes)
        rho_d = eng.xc_rho(X, T, nt, mgga)              # (5, ld)
        del T
        rho = rho_d[:, :nt].cpu().numpy()
        exc, vrho, vsigma, vt = functional.eval(rho)
        exc, v = chain_rule(rho, exc, vrho, vsigma, vt)
        w_h = weights[i0:i1]
        nelec += float((rho[0] * w_h).sum())
        excsum += float((rho[0] * w_h * exc).sum())
        v_d = torch.zeros_like(rho_d)
        v_d[:, :nt] = torch.from_numpy(v).to(dev)
        G = eng.xc_aow(X, v_d, nt, mgga)                # (planes, nao, ld)
        eng.ozaki_k(X[0], G[0], w, out=vmat, accumulate=True)
        for d in range(1, planes):
            eng.ozaki_k(X[d], G[d], w, out=vtau, accumulate=True)
        del X, G
    vmat = vmat + vmat.T
    if mgga:
        # sum_d X_d^T (w o fl32(1/2 vtau X_d)) is symmetric up to the FP32
        # rounding of one operand: its symmetric part keeps vmat exactly
        # symmetric
        vmat += 0.5 * (vtau + vtau.T)
    return nelec, excsum, vmat.cpu().numpy()
