"""FP64 CPU oracle of the COSX path -- TEST INFRASTRUCTURE.

Only tests/, __graft_entry__.smoke() and bench.py's cpu_baseline / reference
arm use this package, and only as the checker or the timed CPU baseline.
The product library never imports, links or calls it.

``build()`` compiles cosx_oracle.c with gcc (-O2 -fopenmp) into
oracle/liboracle.so.  The Python functions below wrap it and add the NumPy
pieces of the reference's K assembly (gpu/sgx_k.py:717-742):

    F = X (proj @ dm),  G = sum_mu A F  (oracle_cosx_g),
    K = X^T (w o G),  K <- proj^T K if sym,  K <- (K + K^T) / 2.

Parity is pinned by tests/test_oracle_golden.py against vectors produced by
the reference's own Python (tests/golden/make_golden.py) and against
closed-form values.
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, 'cosx_oracle.c')
LIB = os.path.join(HERE, 'liboracle.so')

_lib = None


def build(force=False):
    if (not force and os.path.exists(LIB)
            and os.path.getmtime(LIB) >= os.path.getmtime(SRC)):
        return LIB
    cmd = ['gcc', '-O2', '-fopenmp', '-shared', '-fPIC', '-std=c11',
           '-D_DEFAULT_SOURCE', SRC, '-o', LIB + '.tmp', '-lm']
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError('oracle build failed:\n' + res.stderr)
    os.replace(LIB + '.tmp', LIB)
    return LIB


REF_DIR = os.path.join(HERE, '_ref')
REF_GPU_LIB = os.path.join(REF_DIR, 'libref_gpu.so')


def build_ref_gpu(force=False):
    """Compile the reference's extracted CUDA kernels with this directory's
    launchers (ref_gpu/harness.cu) into oracle/_ref/libref_gpu.so, when
    oracle/_ref/ref_kernels.cuh exists; returns the library path or None.
    Test infrastructure: the GPU-side baseline arm of bench.py."""
    src = os.path.join(REF_DIR, 'ref_kernels.cuh')
    harness = os.path.join(HERE, 'ref_gpu', 'harness.cu')
    if not os.path.exists(src):
        return None
    if (not force and os.path.exists(REF_GPU_LIB)
            and os.path.getmtime(REF_GPU_LIB) >= max(os.path.getmtime(src),
                                                     os.path.getmtime(harness))):
        return REF_GPU_LIB
    nvcc = os.path.join(os.environ.get('CUDA_HOME', '/usr/local/cuda'), 'bin', 'nvcc')
    cmd = [nvcc, '-gencode', 'arch=compute_103a,code=sm_103a', '-std=c++14', '-O3',
           '-Xcompiler', '-fPIC', '-shared', '-I', REF_DIR, harness,
           '-o', REF_GPU_LIB + '.tmp']
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError('reference kernel build failed:\n' + res.stderr[-3000:])
    os.replace(REF_GPU_LIB + '.tmp', REF_GPU_LIB)
    return REF_GPU_LIB


def _load():
    global _lib
    if _lib is None:
        build()
        _lib = ctypes.CDLL(LIB)
        P, I, D, I64 = (ctypes.c_void_p, ctypes.c_int, ctypes.c_double,
                        ctypes.c_int64)
        basis = [I, I] + [P] * 9 + [P] * 4
        _lib.oracle_boys.argtypes = [I, D, P]
        _lib.oracle_int3c1e.argtypes = basis + [P, I64, D, P]
        _lib.oracle_cosx_g.argtypes = basis + [P, I64, D, D, P, P]
        _lib.oracle_ao_eval.argtypes = basis + [P, I64, P]
        _lib.oracle_vv10_sum.argtypes = [P, P, P, P, I64, P, P, P]
        _lib.oracle_ao_eval_deriv1.argtypes = basis + [P, I64, P]
        _lib.oracle_pair_keep.argtypes = basis + [D, P]
        _lib.oracle_becke_partition.argtypes = [P, I64, P, P, I, P]
        _lib.oracle_int1e_st.argtypes = basis + [P, P]
        _lib.oracle_hartree.argtypes = basis + [P, I64, P, P]
        for f in ('oracle_boys', 'oracle_int3c1e', 'oracle_cosx_g',
                  'oracle_ao_eval', 'oracle_vv10_sum', 'oracle_ao_eval_deriv1',
                  'oracle_pair_keep', 'oracle_becke_partition', 'oracle_int1e_st',
                  'oracle_hartree'):
            getattr(_lib, f).restype = I
    return _lib


def _p(a):
    return a.ctypes.data_as(ctypes.c_void_p)


class _Basis:
    """Keeps the packed arrays alive for one call."""

    def __init__(self, mol):
        from pyscf_wb97mv_fast_gb300.basis import cart2sph
        pk = mol.packed()
        self.arrays = [pk['atom_coords'], pk['shell_atom'], pk['shell_l'],
                       pk['shell_nprim'], pk['shell_nctr'], pk['shell_exp_off'],
                       pk['shell_coef_off'], pk['exps'], pk['coeffs']]
        self.c2s = [np.ascontiguousarray(cart2sph(l)) for l in range(4)]
        self.args = ([pk['natm'], pk['nbas']] + [_p(a) for a in self.arrays]
                     + [_p(c) for c in self.c2s])
        self.nao = pk['nao']


def boys(nmax, t):
    out = np.zeros(nmax + 1)
    _load().oracle_boys(int(nmax), float(t), _p(out))
    return out


def int3c1e(mol, coords, omega=0.0):
    """(ng, nao, nao) FP64 dense integrals at absolute coordinates."""
    b = _Basis(mol)
    c = np.ascontiguousarray(coords, dtype=np.float64)
    out = np.zeros((len(c), b.nao, b.nao))
    _load().oracle_int3c1e(*b.args, _p(c), len(c), float(omega), _p(out))
    return out


def cosx_g(mol, coords, F, omega=0.0, pair_cutoff=1e-14):
    """G (ng, nao) FP64 for F (ng, nao)."""
    b = _Basis(mol)
    c = np.ascontiguousarray(coords, dtype=np.float64)
    F = np.ascontiguousarray(F, dtype=np.float64)
    G = np.zeros_like(F)
    _load().oracle_cosx_g(*b.args, _p(c), len(c), float(omega),
                          float(pair_cutoff), _p(F), _p(G))
    return G


def becke_partition(points, owner, atom_coords):
    """Owner-atom Becke weights (FP64), the grid builder's partition
    without the product library."""
    pts = np.ascontiguousarray(points, dtype=np.float64)
    own = np.ascontiguousarray(owner, dtype=np.int32)
    at = np.ascontiguousarray(atom_coords, dtype=np.float64)
    out = np.empty(len(pts))
    if _load().oracle_becke_partition(_p(pts), len(pts), _p(own), _p(at),
                                      len(at), _p(out)) != 0:
        raise MemoryError('oracle_becke_partition')
    return out


def int1e(mol):
    """(S, T, V) FP64 (nao, nao): overlap, kinetic energy and the nuclear
    attraction of the molecule's own nuclei (V from the dense 3-centre
    integrals at the nuclei)."""
    b = _Basis(mol)
    S = np.zeros((b.nao, b.nao))
    T = np.zeros((b.nao, b.nao))
    _load().oracle_int1e_st(*b.args, _p(S), _p(T))
    xyz = np.ascontiguousarray(mol.atom_coords(), dtype=np.float64)
    A = int3c1e(mol, xyz)
    V = -np.einsum('c,cmn->mn', np.asarray(mol.atom_charges(), dtype=np.float64), A)
    return S, T, V


def hartree(mol, coords, dm):
    """v_H(g) = sum D_{mu nu} (mu nu | 1/|r - g|), FP64, every pair."""
    b = _Basis(mol)
    c = np.ascontiguousarray(coords, dtype=np.float64)
    D = np.ascontiguousarray(dm, dtype=np.float64)
    v = np.zeros(len(c))
    _load().oracle_hartree(*b.args, _p(c), len(c), _p(D), _p(v))
    return v


def pair_keep(mol, pair_cutoff=1e-14):
    """(nbas, nbas) bool, lower triangle: the shell pairs the reference's
    magnitude cut keeps (gpu/shellpairs.py:287-294)."""
    b = _Basis(mol)
    n = len(mol.shells)
    keep = np.zeros((n, n), dtype=np.uint8)
    if _load().oracle_pair_keep(*b.args, float(pair_cutoff), _p(keep)) != 0:
        raise MemoryError('oracle_pair_keep')
    return keep.astype(bool)


def model_flops_per_point(mol, pair_cutoff=1e-14):
    """(model flops per grid point, kept pairs): the work the CPU baselines
    are credited with, from the pure-Python flop model over the shell pairs
    the oracle keeps.  A generally contracted shell counts once per
    contraction column, as in the GPU kernels' work count."""
    from pyscf_wb97mv_fast_gb300.flops_model import task_flops
    keep = pair_keep(mol, pair_cutoff)
    shells = mol.shells
    total, npairs, cache = 0, 0, {}
    for i, si in enumerate(shells):
        for j in range(i + 1):
            if not keep[i, j]:
                continue
            sj = shells[j]
            for ci in range(si.nctr):
                for cj in range(sj.nctr if j < i else ci + 1):
                    diag = j == i and cj == ci
                    key = (si.l, sj.l, si.nprim, sj.nprim, diag)
                    v = cache.get(key)
                    if v is None:
                        v = cache[key] = task_flops(*key)
                    total += v
                    npairs += 1
    return float(total), npairs


def ao_eval(mol, coords):
    """X (ng, nao) FP64."""
    b = _Basis(mol)
    c = np.ascontiguousarray(coords, dtype=np.float64)
    X = np.zeros((len(c), b.nao))
    _load().oracle_ao_eval(*b.args, _p(c), len(c), _p(X))
    return X


def ao_eval_deriv1(mol, coords):
    """X and gradients (4, ng, nao) FP64."""
    b = _Basis(mol)
    c = np.ascontiguousarray(coords, dtype=np.float64)
    X = np.zeros((4, len(c), b.nao))
    _load().oracle_ao_eval_deriv1(*b.args, _p(c), len(c), _p(X))
    return X


def nlc_vxc(mol, coords, weights, dm, nlc_coefs, thresh=1e-8):
    """FP64 restatement of the reference's VV10 flow (gpu/vv10.py:268-342 =
    NumInt.nr_nlc_vxc): (nelec, excsum, vmat); nlc_coefs [((b, C), fac)]."""
    import math
    ao = ao_eval_deriv1(mol, coords)
    w = np.asarray(weights, dtype=np.float64)
    T = ao[0] @ dm
    rho0 = (T * ao[0]).sum(axis=1)
    grad = 2.0 * np.einsum('pm,dpm->dp', T, ao[1:4])
    nelec = float((rho0 * w).sum())
    n = len(w)
    exc, v0, v1 = np.zeros(n), np.zeros(n), np.zeros(n)
    for (Bvv, Cvv), fac in nlc_coefs:
        ind = rho0 >= thresh
        R, gr = rho0[ind], grad[:, ind]
        pi43 = 4.0 * math.pi / 3.0
        Kvv = Bvv * 1.5 * math.pi * (9.0 * math.pi) ** (-1.0 / 6.0)
        Beta = ((3.0 / (Bvv * Bvv)) ** 0.75) / 32.0
        G = (gr ** 2).sum(axis=0)
        W0tmp = Cvv * (G / (R * R)) ** 2
        W0 = np.sqrt(W0tmp + pi43 * R)
        dW0dR = (0.5 * pi43 * R - 2.0 * W0tmp) / W0
        dW0dG = W0tmp * R / (G * W0)
        kappa = Kvv * R ** (1.0 / 6.0)
        dKdR = kappa / 6.0
        q = R * w[ind]
        F, U, W = vv10_sum(coords[ind], q, W0, kappa)
        exc[ind] += fac * (Beta + 0.5 * F)
        v0[ind] += fac * (Beta + F + 1.5 * (U * dKdR + W * dW0dR))
        v1[ind] += fac * (1.5 * W * dW0dG)
    excsum = float((rho0 * w * exc).sum())
    wv = np.empty((4, n))
    wv[0] = 0.5 * v0 * w
    wv[1:4] = 2.0 * v1[None] * grad * w[None]
    aow = np.einsum('dpm,dp->pm', ao, wv)
    vmat = ao[0].T @ aow
    return nelec, excsum, vmat + vmat.T


def xc_chain_rule(rho, exc, vrho, vsigma, vtau):
    """libxc derivatives -> density-parameter derivatives v (5, P): vrho,
    2 vsigma grad rho, vtau (reference gpu/xc.py:96-116; zero rows for an
    absent vsigma / vtau)."""
    v = np.zeros((5, rho.shape[1]))
    v[0] = vrho
    if vsigma is not None:
        v[1:4] = 2.0 * np.asarray(vsigma)[None] * rho[1:4]
    if vtau is not None:
        v[4] = vtau
    return np.asarray(exc, dtype=np.float64), v


def nr_rks(mol, coords, weights, dm, functional, xctype, ao=None):
    """FP64 restatement of the reference's semilocal XC flow
    (gpu/xc.py:130-201 = NumInt.nr_rks for one RKS density):
    (nelec, excsum, vmat).  functional.eval(rho (5, P)) returns (exc, vrho,
    vsigma, vtau) in the libxc convention; xctype 'LDA', 'GGA' or 'MGGA';
    ao: the AO values and gradients (4, P, nao) when already evaluated."""
    if ao is None:
        ao = ao_eval_deriv1(mol, coords)
    w = np.asarray(weights, dtype=np.float64)
    n = len(w)
    T = ao[0] @ dm
    rho = np.zeros((5, n))
    rho[0] = (T * ao[0]).sum(axis=1)
    rho[1:4] = 2.0 * np.einsum('pm,dpm->dp', T, ao[1:4])
    if xctype == 'MGGA':
        for d in range(1, 4):
            rho[4] += 0.5 * ((ao[d] @ dm) * ao[d]).sum(axis=1)
    exc, vrho, vsigma, vtau = functional.eval(rho)
    exc, v = xc_chain_rule(rho, exc, vrho, vsigma, vtau)
    nelec = float((rho[0] * w).sum())
    excsum = float((rho[0] * w * exc).sum())
    wv = v * w[None]
    wv[0] *= 0.5
    aow = np.einsum('dpm,dp->pm', ao, wv[:4])
    vmat = ao[0].T @ aow
    vmat = vmat + vmat.T
    if xctype == 'MGGA':
        wtau = 0.5 * wv[4]
        for d in range(1, 4):
            vmat += (ao[d] * wtau[:, None]).T @ ao[d]
    return nelec, excsum, vmat


def vv10_sum(coords, q, w0, kappa):
    """FP64 brute-force F (x -1.5), U, W."""
    c = np.ascontiguousarray(coords, dtype=np.float64)
    q, w0, kappa = (np.ascontiguousarray(a, dtype=np.float64)
                    for a in (q, w0, kappa))
    n = len(q)
    F, U, W = np.zeros(n), np.zeros(n), np.zeros(n)
    _load().oracle_vv10_sum(_p(c), _p(q), _p(w0), _p(kappa), n, _p(F), _p(U),
                            _p(W))
    return F, U, W


def cosx_k(mol, coords, weights, dm, omega=0.0, proj=None, sym=False,
           hermi=1, return_parts=False):
    """FP64 COSX K of the reference's get_k (gpu/sgx_k.py:709-742) on a grid
    (absolute coordinates): no screening, no FP32 rounding anywhere."""
    X = ao_eval(mol, coords)
    nao = X.shape[1]
    proj = np.eye(nao) if proj is None else np.asarray(proj)
    F = X @ (proj @ dm)
    G = cosx_g(mol, coords, F, omega)
    K = X.T @ (np.asarray(weights)[:, None] * G)
    if sym:
        K = proj.T @ K
    if hermi == 1:
        K = (K + K.T) * 0.5
    if return_parts:
        return K, X, F, G
    return K


# -- the reference's FP64 screening bound (test aid) --------------------------

_BOUND_ETA = 0.25


def _c2s_tau(l):
    """max over spherical columns of sum over Cartesians |c2s| (the
    reference's per-shell tau, gpu/shellpairs.py:220)."""
    from pyscf_wb97mv_fast_gb300.basis import cart2sph
    return float(np.abs(cart2sph(l)).sum(axis=0).max())


def _bound_c_grid(la, lb, p, rpa, rpb):
    """C_ab = sup_{s >= 0} (s + |PA|)^la (s + |PB|)^lb exp(-eta p s^2) as the
    reference finds it (gpu/shellpairs.py:123-168): the maximum over 4097
    equally spaced s in [0, s_max], s_max where the envelope has fallen
    below 1e-30 of its scale, times 1.01; la = lb = 0 gives 1."""
    if la == 0 and lb == 0:
        return np.ones_like(p)
    L = float(la + lb)
    rmax = np.maximum(rpa, rpb)
    s = np.sqrt(np.maximum(0.0, (L * np.log(rmax + 1.0) + 69.0) / (_BOUND_ETA * p)))
    for _ in range(8):
        s = np.sqrt(np.maximum(0.0, (L * np.log(np.maximum(s, 1e-300) + rmax) + 69.0)
                               / (_BOUND_ETA * p)))
    x = np.linspace(0.0, 1.0, 4097)[:, None] * (1.05 * s)[None, :]
    f = (x + rpa) ** la * (x + rpb) ** lb * np.exp(-_BOUND_ETA * p * x * x)
    return f.max(axis=0) * 1.01


def screen_pairs_fp64(mol, pair_cutoff=1e-14):
    """Per kept shell pair (ish >= jsh): (ish, jsh, P (m, 3), p' (m,),
    pref (m,), tau) over its primitive pairs, the data of the reference's
    locked bound (gpu/shellpairs.py:286-370): pref = cmax_a cmax_b K_AB C_ab
    2 pi / p', p' = 0.75 p, tau = tau_l(ish) tau_l(jsh)."""
    keep = pair_keep(mol, pair_cutoff)
    shells = mol.shells
    xyz = mol.atom_coords()
    out = []
    for i, si in enumerate(shells):
        A = xyz[si.atom]
        ca = np.abs(np.asarray(si.coeffs).reshape(si.nprim, si.nctr)).max(axis=1)
        for j in range(i + 1):
            if not keep[i, j]:
                continue
            sj = shells[j]
            B = xyz[sj.atom]
            cb = np.abs(np.asarray(sj.coeffs).reshape(sj.nprim, sj.nctr)).max(axis=1)
            al = np.repeat(np.asarray(si.exps, dtype=np.float64), sj.nprim)
            be = np.tile(np.asarray(sj.exps, dtype=np.float64), si.nprim)
            cab = np.repeat(ca, sj.nprim) * np.tile(cb, si.nprim)
            p = al + be
            P = (al[:, None] * A + be[:, None] * B) / p[:, None]
            K = np.exp(-al * be / p * float(((A - B) ** 2).sum()))
            C = _bound_c_grid(si.l, sj.l, p, np.linalg.norm(P - A, axis=1),
                              np.linalg.norm(P - B, axis=1))
            pp = (1.0 - _BOUND_ETA) * p
            out.append((i, j, P, pp, cab * K * C * (2.0 * np.pi / pp),
                        _c2s_tau(si.l) * _c2s_tau(sj.l)))
    return out


def screen_keep_fp64(mol, coords, weights, F, tol, block_pts=32,
                     pair_cutoff=1e-14):
    """The reference's host screen (GpuKBuilder._kept_host,
    gpu/sgx_k.py:926-958) in FP64: keep (nblk, npairs) bool for blocks of
    block_pts consecutive points, where tau sum_prim pref F0(p' d^2) times
    max_g w_g max(sum_{t in A} |F_gt|, sum_{t in B} |F_gt|) >= tol, with d
    the distance of P from the block centroid less the block radius
    (gpu/shellpairs.py:545-555).  Returns (keep, [(ish, jsh), ...])."""
    from scipy.special import erf
    coords = np.asarray(coords, dtype=np.float64)
    w = np.asarray(weights, dtype=np.float64)
    F = np.asarray(F, dtype=np.float64)
    ng = len(coords)
    nblk = -(-ng // block_pts)
    ao_loc = mol.packed()['ao_loc']
    fw = np.abs(F) * w[:, None]
    seg = np.add.reduceat(fw, ao_loc[:-1], axis=1)           # (ng, nbas)
    msh = np.zeros((nblk, seg.shape[1]))
    cen = np.zeros((nblk, 3))
    rad = np.zeros(nblk)
    for b in range(nblk):
        sl = slice(b * block_pts, min(ng, (b + 1) * block_pts))
        msh[b] = seg[sl].max(axis=0)
        cen[b] = coords[sl].mean(axis=0)
        rad[b] = np.linalg.norm(coords[sl] - cen[b], axis=1).max()
    pairs = screen_pairs_fp64(mol, pair_cutoff)
    keep = np.zeros((nblk, len(pairs)), dtype=bool)
    for k, (i, j, P, pp, pref, tau) in enumerate(pairs):
        d = np.linalg.norm(P[None, :, :] - cen[:, None, :], axis=2) - rad[:, None]
        T = pp[None, :] * np.maximum(d, 0.0) ** 2
        Ts = np.maximum(T, 1e-300)
        f0 = np.where(T > 1e-14, 0.5 * np.sqrt(np.pi / Ts) * erf(np.sqrt(Ts)), 1.0)
        bound = tau * (f0 * pref[None, :]).sum(axis=1)
        keep[:, k] = bound * np.maximum(msh[:, i], msh[:, j]) >= tol
    return keep, [(i, j) for (i, j, *_rest) in pairs]
