"""VV10 non-local correlation on the GPU (reference:
pyscf_wb97mv_fast/gpu/vv10.py).

* ``Vv10Kernel.kernel_sum(coords, q, W0, kappa) -> (F, U, W)``: the
  O(N_g^2) double sum through the native tiled kernel (FP32 pair terms,
  Kahan inside a 256-point tile, FP64 across tiles, device-side tile-pair
  pruning when tile_tol > 0).  F is returned as -1.5 x the raw sum, the
  libdft VXC_vv10nlc convention the reference follows (:216-221).
* ``vv10_pointwise``: the per-point FP64 quantities of PySCF's _vv10nlc
  (reference :243-265), in torch on the device.
* ``gpu_nr_nlc_vxc``: same signature and result as
  ``NumInt.nr_nlc_vxc`` -> (nelec, excsum, vmat) (reference :268-342): AO
  values and gradients (FP64, native), GGA density, threshold
  rho >= 1e-8, pointwise terms, kernel_sum, the GGA potential and the Fock
  contraction vmat = X^T (w v) X + transpose, all on the device in FP64
  except the pair sum.
"""
import math

import numpy as np

from pyscf_wb97mv_fast_gb300 import _native
from pyscf_wb97mv_fast_gb300.cosx import CosxEngine, as_molecule

THRESH = 1e-8
Unsupported = _native.Unsupported


def _torch():
    import torch
    return torch


class Vv10Kernel:
    """The double sum; tile_tol > 0 enables device-side tile-pair pruning."""

    def __init__(self, tile_tol=0.0):
        self.tile_tol = float(tile_tol)
        self.last_pairs_kept = None

    def kernel_sum(self, coords, q, W0, kappa):
        """coords (P, 3), q, W0, kappa (P,) on the device -> F, U, W FP64."""
        torch = _torch()
        _check_points(coords, 'coords')
        dev = coords.device
        n = int(coords.shape[0])
        F = torch.zeros(n, dtype=torch.float64, device=dev)
        U = torch.zeros_like(F)
        W = torch.zeros_like(F)
        if n == 0:
            self.last_pairs_kept = (0, 0)
            return F, U, W
        xyz = coords.to(torch.float32).contiguous()
        q32, w32, k32 = (_per_point(a, n, dev, name) for a, name in
                         ((q, 'q'), (W0, 'W0'), (kappa, 'kappa')))
        kept = _native.ctypes.c_int64()
        stream = _native.ctypes.c_void_p(torch.cuda.current_stream(dev).cuda_stream)
        _native.check(_native.lib().wb_vv10_kernel_sum(
            _native.ptr(xyz), _native.ptr(q32), _native.ptr(w32), _native.ptr(k32),
            n, self.tile_tol, _native.ptr(F), _native.ptr(U), _native.ptr(W),
            stream, _native.ctypes.byref(kept)), 'wb_vv10_kernel_sum')
        self.last_pairs_kept = (int(kept.value), n * n)
        return F, U, W


    def kernel_sum_batch(self, coords, q, W0, kappa):
        """The double sums of several molecules in one launch: lists of
        per-molecule device arrays as kernel_sum takes them -> lists of F,
        U, W (each molecule's sums over its own points only; bitwise equal
        to kernel_sum per molecule)."""
        torch = _torch()
        if not coords or not len(coords) == len(q) == len(W0) == len(kappa):
            raise ValueError('one coords, q, W0 and kappa array per molecule')
        for c in coords:
            _check_points(c, 'coords')
        sizes = [int(c.shape[0]) for c in coords]
        dev = coords[0].device
        if any(c.device != dev for c in coords):
            raise ValueError('coords of one batch must share a device')
        offsets = np.concatenate([[0], np.cumsum(sizes)]).astype(np.int64)
        n = int(offsets[-1])
        xyz = torch.cat([c.to(torch.float32) for c in coords]).contiguous()
        q32, w32, k32 = (torch.cat([_per_point(a, m, dev, name)
                                    for a, m in zip(arrs, sizes)]).contiguous()
                         for arrs, name in ((q, 'q'), (W0, 'W0'), (kappa, 'kappa')))
        F = torch.zeros(n, dtype=torch.float64, device=dev)
        U = torch.zeros_like(F)
        W = torch.zeros_like(F)
        kept = _native.ctypes.c_int64()
        stream = _native.ctypes.c_void_p(torch.cuda.current_stream(dev).cuda_stream)
        _native.check(_native.lib().wb_vv10_kernel_sum_batch(
            len(sizes), offsets.ctypes.data_as(_native.ctypes.c_void_p),
            _native.ptr(xyz), _native.ptr(q32), _native.ptr(w32), _native.ptr(k32),
            self.tile_tol, _native.ptr(F), _native.ptr(U), _native.ptr(W), stream,
            _native.ctypes.byref(kept)), 'wb_vv10_kernel_sum_batch')
        self.last_pairs_kept = (int(kept.value), int(sum(m * m for m in sizes)))
        sl = [slice(int(offsets[i]), int(offsets[i + 1])) for i in range(len(sizes))]
        return [F[x] for x in sl], [U[x] for x in sl], [W[x] for x in sl]


def _check_points(coords, name):
    """coords must be an (n, 3) torch tensor on a CUDA device: the kernels
    read its raw pointer."""
    torch = _torch()
    if not isinstance(coords, torch.Tensor) or not coords.is_cuda:
        raise ValueError('%s must be a torch tensor on a CUDA device' % name)
    if coords.dim() != 2 or coords.shape[1] != 3:
        raise ValueError('%s has shape %s, expected (n, 3)'
                         % (name, tuple(coords.shape)))


def _per_point(a, n, dev, name):
    """A per-point array (n,) as contiguous FP32 on dev."""
    torch = _torch()
    t = torch.as_tensor(a, device=dev).to(torch.float32).contiguous()
    if t.dim() != 1 or t.shape[0] != n:
        raise ValueError('%s has shape %s, expected (%d,)' % (name, tuple(t.shape), n))
    return t


def vv10_pointwise(rho0, grad, weights, nlc_pars):
    """Per-point FP64 terms on the thresholded set: q, W0, kappa, dW0/dR,
    dW0/dG, dK/dR, Beta (torch tensors; Beta a float)."""
    Bvv, Cvv = nlc_pars
    pi = math.pi
    pi43 = 4.0 * pi / 3.0
    Kvv = Bvv * 1.5 * pi * (9.0 * pi) ** (-1.0 / 6.0)
    Beta = ((3.0 / (Bvv * Bvv)) ** 0.75) / 32.0
    R = rho0
    G = (grad ** 2).sum(dim=0)
    W0tmp = Cvv * (G / (R * R)) ** 2
    W0 = (W0tmp + pi43 * R).sqrt()
    dW0dR = (0.5 * pi43 * R - 2.0 * W0tmp) / W0
    dW0dG = W0tmp * R / (G * W0)
    kappa = Kvv * R ** (1.0 / 6.0)
    dKdR = kappa / 6.0
    q = R * weights
    return q, W0, kappa, dW0dR, dW0dG, dKdR, Beta


class Vv10Context:
    """Per-mf state of the VV10 flow: the native engine (AO tables) and the
    kernel-sum settings."""

    def __init__(self, mol, tile_tol=0.0, device=None):
        self.mol = mol
        self.tile_tol = float(tile_tol)
        self.device = device
        self.engine = None
        self.kernel = Vv10Kernel(tile_tol)

    def build(self):
        if self.engine is None:
            self.engine = CosxEngine(as_molecule(self.mol), device=self.device)
        return self.engine


def _prepare_dm(dm, hermi):
    dm = np.asarray(dm, dtype=np.float64)
    if dm.ndim == 3 and dm.shape[0] == 1:
        dm = dm[0]
    if dm.ndim != 2 or dm.shape[0] != dm.shape[1]:
        raise Unsupported(_native.WB_ERR_UNSUPPORTED,
                          'GPU VV10 supports a single RKS density matrix')
    if hermi != 1:
        dm = 0.5 * (dm + dm.T)
    return dm


def vv10_prepare(eng, g, D, nlc_pars, gemm='fp64'):
    """The steps of vv10_energy_fock before the double sum (the GGA density
    on the NLC grid g, the threshold and the pointwise terms): a state for
    vv10_finish; st['xyz'], st['q'], st['W0'], st['kappa'] are the double
    sum's inputs (Vv10Kernel.kernel_sum or, for several molecules,
    kernel_sum_batch).  gemm as in vv10_energy_fock."""
    torch = _torch()
    if gemm not in ('fp64', 'split64', 'fp32'):
        raise ValueError("gemm must be 'fp64', 'split64' or 'fp32'")
    n = g.n
    ao = g.X[:, :, :n]
    w = g.weights
    if gemm == 'fp32':
        T = eng.ozaki_f(g.X[0], D)[:, :n].to(torch.float64)
    elif gemm == 'split64':
        T = eng.ozaki_f(g.X[0], D, fp64=True)[:, :n]
    else:
        T = D @ ao[0]
    rho0 = (T * ao[0]).sum(dim=0)
    grad = 2.0 * torch.einsum('mp,dmp->dp', T, ao[1:4])
    ind = rho0 >= THRESH
    q, W0, kappa, dW0dR, dW0dG, dKdR, Beta = vv10_pointwise(
        rho0[ind], grad[:, ind], w[ind], nlc_pars)
    return dict(eng=eng, g=g, gemm=gemm, n=n, rho0=rho0, grad=grad, ind=ind,
                xyz=g.coords[ind].to(torch.float32), q=q, W0=W0, kappa=kappa,
                dW0dR=dW0dR, dW0dG=dW0dG, dKdR=dKdR, Beta=Beta)


def vv10_finish(st, F, U, W):
    """E_nl and V_nl from a vv10_prepare state and the double sums F, U, W
    of its points."""
    torch = _torch()
    g, n, ind, w = st['g'], st['n'], st['ind'], st['g'].weights
    ao = g.X[:, :, :n]
    Beta = st['Beta']
    dev = st['rho0'].device
    exc = torch.zeros(n, dtype=torch.float64, device=dev)
    v0 = torch.zeros_like(exc)
    v1 = torch.zeros_like(exc)
    exc[ind] = Beta + 0.5 * F
    v0[ind] = Beta + F + 1.5 * (U * st['dKdR'] + W * st['dW0dR'])
    v1[ind] = 1.5 * W * st['dW0dG']
    e_nl = (st['rho0'] * w * exc).sum()
    grad = st['grad']
    if st['gemm'] != 'fp64':
        # G = 1/2 v0 X0 + sum_d 2 v1 grad_d X_d, then X0^T (w o G), G FP64
        # or rounded once to FP32
        vv = torch.empty((4, n), dtype=torch.float64, device=dev)
        vv[0] = 0.5 * v0
        vv[1:4] = 2.0 * v1[None, :] * grad
        dt = torch.float32 if st['gemm'] == 'fp32' else torch.float64
        G = torch.zeros_like(g.X[0], dtype=dt)
        G[:, :n] = torch.einsum('dmp,dp->mp', ao, vv).to(dt)
        vmat = st['eng'].ozaki_k(g.X[0], G, w)
        return e_nl, vmat + vmat.T
    wv = torch.empty((4, n), dtype=torch.float64, device=dev)
    wv[0] = 0.5 * v0 * w
    wv[1:4] = 2.0 * v1[None, :] * grad * w[None, :]
    aow = torch.einsum('dmp,dp->mp', ao, wv)
    vmat = ao[0] @ aow.T
    return e_nl, vmat + vmat.T


def vv10_energy_fock(eng, g, D, nlc_pars, kernel=None, fp32=False, gemm='fp64'):
    """E_nl and V_nl of one density on a device grid, all on the device:
    g holds coordinates (engine frame), weights and the deriv-1 AO values
    X (4, nao, ld) (scf.DeviceGrid); D (nao, nao) FP64 device.  The same
    steps as gpu_nr_nlc_vxc for one parameter set (b, C) with factor 1:
    GGA density, threshold rho >= 1e-8, pointwise terms, the pair sum, the
    GGA potential and vmat = X^T (w v) X + transpose.  Returns (E_nl
    device scalar, V_nl (nao, nao)).  The two GEMMs (D X and the Fock
    side) run as gemm:
      'fp64'    plain FP64 GEMMs;
      'split64' the bf16 Ozaki split with FP64 operands and results (42
                bits of the per-row / per-column maxima), the SCF's FP64
                tail;
      'fp32'    the split with D X rounded once to FP32 and the Fock side
                from an FP32-rounded G, the SCF's FP32 stages (fp32=True
                is the same)."""
    st = vv10_prepare(eng, g, D, nlc_pars, 'fp32' if fp32 else gemm)
    kernel = kernel or Vv10Kernel(0.0)
    F, U, W = kernel.kernel_sum(st['xyz'], st['q'], st['W0'], st['kappa'])
    return vv10_finish(st, F, U, W)


def gpu_nr_nlc_vxc(ctx, ni, mol, grids, xc_code, dm, relativity=0, hermi=1,
                   max_memory=2000, verbose=None):
    """GPU replacement of NumInt.nr_nlc_vxc (RKS ground state)."""
    torch = _torch()
    if relativity not in (0, None):
        raise Unsupported(_native.WB_ERR_UNSUPPORTED,
                          'relativistic NLC not supported')
    dm = _prepare_dm(dm, hermi)
    nlc_coefs = ni.nlc_coeff(xc_code)
    if not nlc_coefs:
        raise Unsupported(_native.WB_ERR_UNSUPPORTED,
                          '%r has no NLC parameter set' % (xc_code,))
    eng = ctx.build()
    dev = eng.device
    nao = eng.nao
    coords = eng.relative(np.asarray(grids.coords, dtype=np.float64))
    w = torch.as_tensor(np.asarray(grids.weights, dtype=np.float64), device=dev)
    n = int(coords.shape[0])
    ao = eng.ao_eval_deriv1(coords)[:, :, :n]             # (4, nao, n)
    D = torch.as_tensor(dm, device=dev)
    T = D @ ao[0]                                         # (nao, n)
    rho0 = (T * ao[0]).sum(dim=0)
    grad = 2.0 * torch.einsum('mp,dmp->dp', T, ao[1:4])
    nelec = float((rho0 * w).sum())
    exc = torch.zeros(n, dtype=torch.float64, device=dev)
    v0 = torch.zeros_like(exc)
    v1 = torch.zeros_like(exc)
    c32 = coords.to(torch.float32)
    for nlc_pars, fac in nlc_coefs:
        ind = rho0 >= THRESH
        q, W0, kappa, dW0dR, dW0dG, dKdR, Beta = vv10_pointwise(
            rho0[ind], grad[:, ind], w[ind], nlc_pars)
        F, U, W = ctx.kernel.kernel_sum(c32[ind], q, W0, kappa)
        exc[ind] += fac * (Beta + 0.5 * F)
        v0[ind] += fac * (Beta + F + 1.5 * (U * dKdR + W * dW0dR))
        v1[ind] += fac * (1.5 * W * dW0dG)
    excsum = float((rho0 * w * exc).sum())
    wv = torch.empty((4, n), dtype=torch.float64, device=dev)
    wv[0] = 0.5 * v0 * w                                  # *.5 for vmat + vmat^T
    wv[1:4] = 2.0 * v1[None, :] * grad * w[None, :]
    aow = torch.einsum('dmp,dp->mp', ao, wv)
    vmat = ao[0] @ aow.T
    vmat = vmat + vmat.T
    return nelec, excsum, vmat.cpu().numpy()
