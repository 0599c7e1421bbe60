"""Generates the golden fixtures of tests/golden/ by running the reference's
own Python (Cedrus810/pyscf-wb97mv-fast: a checkout of it, named by the
first argument or by WB_REFERENCE_ROOT) on this project's synthetic
molecules.

PySCF is not installed, so the few PySCF names the reference modules import
are stubbed: ``pyscf.gto.mole.cart2sph`` is served by this project's
``basis.cart2sph`` (the spherical convention is therefore this project's in
both codes) and the Mole accessors by ``basis.Molecule``.  Everything else --
Boys (gpu/boys.py), the shell-pair data, Hermite and R recurrences and
contracted integrals (gpu/shellpairs.py int3c1e_reference, pair_bound), the
FP64 AO evaluation (gpu/ao_eval.py) and the VV10 kernel sum
(gpu/vv10.py Vv10Kernel, NumPy path) -- is the reference's code, unmodified.

Run from the repository root:
    python tests/golden/make_golden.py <reference checkout> [--only-drugs]
The output files are committed; tests never read the reference.
"""
import os
import sys
import types

import numpy as np


def _reference_root():
    args = [a for a in sys.argv[1:] if not a.startswith('--')]
    root = args[0] if args else os.environ.get('WB_REFERENCE_ROOT', '')
    if not root or not os.path.isdir(os.path.join(root, 'pyscf_wb97mv_fast')):
        raise SystemExit('usage: make_golden.py <reference checkout> '
                         '(or set WB_REFERENCE_ROOT)')
    return root


HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from pyscf_wb97mv_fast_gb300.basis import Molecule, cart2sph  # noqa: E402
from pyscf_wb97mv_fast_gb300.systems import water_dimer  # noqa: E402


def install_stubs(ref_root):
    pyscf = types.ModuleType('pyscf')
    gto = types.ModuleType('pyscf.gto')
    mole = types.ModuleType('pyscf.gto.mole')
    mole.cart2sph = cart2sph
    eval_gto = types.ModuleType('pyscf.gto.eval_gto')
    eval_gto.BLKSIZE = 56
    lib = types.ModuleType('pyscf.lib')
    logger = types.ModuleType('pyscf.lib.logger')
    logger.debug1 = lambda *a, **k: None
    lib.logger = logger
    gto.mole = mole
    gto.eval_gto = eval_gto
    pyscf.gto = gto
    pyscf.lib = lib
    for name, mod in (('pyscf', pyscf), ('pyscf.gto', gto),
                      ('pyscf.gto.mole', mole), ('pyscf.gto.eval_gto', eval_gto),
                      ('pyscf.lib', lib), ('pyscf.lib.logger', logger)):
        sys.modules[name] = mod
    # gpu/xc.py pulls in libxc plumbing; only its Unsupported and
    # _prepare_dm are used by the modules below
    xc = types.ModuleType('pyscf_wb97mv_fast.gpu.xc')

    class Unsupported(Exception):
        pass

    def _prepare_dm(dm, hermi):
        return np.asarray(dm)
    xc.Unsupported = Unsupported
    xc._prepare_dm = _prepare_dm
    sys.modules['pyscf_wb97mv_fast.gpu.xc'] = xc
    sys.path.insert(0, ref_root)


class RefMol:
    """The Mole accessors the reference reads, over a Molecule."""

    def __init__(self, mol):
        self.m = mol
        self.cart = False
        self.nbas = mol.nbas
        self.nao = mol.nao
        self._bas = mol._bas

    def __getattr__(self, name):
        return getattr(self.m, name)


def points(mol, rng, n):
    span = np.abs(mol.atom_coords()).max() + 3.0
    pts = rng.uniform(-span, span, (n, 3))
    far = np.array([[60.0, 0.0, 0.0], [0.0, -45.0, 20.0]])
    return np.vstack([mol.atom_coords(), far, pts])


def write_drugs(ref_root):
    """The reference's six validation geometries (benchmarks/systems/drugs/
    *.xyz, README.md:118-128) as symbols and Angstrom coordinates, read with
    this project's XYZ reader."""
    from pyscf_wb97mv_fast_gb300.systems import read_xyz
    ddir = os.path.join(ref_root, 'benchmarks', 'systems', 'drugs')
    out = {}
    for name in sorted(os.listdir(ddir)):
        if not name.endswith('.xyz'):
            continue
        atoms = read_xyz(os.path.join(ddir, name))
        tag = name[:-4]
        out[tag + '_symbols'] = np.array([a[0] for a in atoms])
        out[tag + '_coords'] = np.array([a[1] for a in atoms], dtype=np.float64)
    np.savez_compressed(os.path.join(HERE, 'drugs.npz'), **out)


def main():
    root = _reference_root()
    if '--only-drugs' in sys.argv:
        write_drugs(root)
        return
    write_drugs(root)
    install_stubs(root)
    from pyscf_wb97mv_fast.gpu import boys as rboys
    from pyscf_wb97mv_fast.gpu import shellpairs as rsp
    from pyscf_wb97mv_fast.gpu import ao_eval as rao
    from pyscf_wb97mv_fast.gpu import vv10 as rvv

    out = {}
    # -- Boys: reference FP64 values and its FP32 Taylor table -----------------
    T = np.concatenate([[0.0, 1e-30, 1e-8], np.linspace(0.0, 50.0, 401),
                        np.geomspace(50.0, 1e6, 41)])
    out['boys_T'] = T
    out['boys_ref'] = np.stack([rboys.boys_ref(n, T) for n in range(7)])
    c_hi, c0_lo = rboys._build_table()
    out['boys_table_hi'] = c_hi
    out['boys_table_c0lo'] = c0_lo
    np.savez_compressed(os.path.join(HERE, 'boys.npz'), **out)

    # -- integrals, bounds, AO values on synthetic molecules -------------------
    cases = [('svp', Molecule.build(water_dimer(), 'synthetic-svp'), 14),
             ('tzvp', Molecule.build(water_dimer(), 'synthetic-tzvp'), 4),
             ('gen', Molecule.build(water_dimer(), 'synthetic-svp',
                                    gen_contract=True), 6)]
    for tag, mol, npts in cases:
        rng = np.random.default_rng(11)
        pts = points(mol, rng, npts)
        rm = RefMol(mol)
        pairs = rsp.ShellPairs(rm)
        res = {'coords': pts, 'atom_coords': mol.atom_coords()}
        for omega in (0.0, 0.3):
            res['A_w%g' % omega] = rsp.int3c1e_reference(pairs, pts, omega=omega)
        blocks = [pts[:8], mol.atom_coords()[0] + rng.normal(scale=0.05, size=(32, 3)),
                  np.array([25.0, 0.0, 0.0]) + rng.normal(scale=1.0, size=(32, 3))]
        for k, blk in enumerate(blocks):
            res['bound_block%d' % k] = blk
            res['bound%d' % k] = rsp.pair_bound(pairs, blk)
        res['pair_rows'] = pairs.pair_rows
        aopts = np.vstack([pts, rng.normal(scale=2.5, size=(40, 3))])
        origin = mol.atom_coords().mean(axis=0)
        pack = rao.ShellPack(rm, origin=origin)
        ev = rao.AoEvaluator(rm, np, pack=pack, mem_budget=1 << 28,
                             dtype='float64', verify=False)
        res['ao_coords'] = aopts
        res['ao'] = ev.eval(aopts - origin, np.arange(mol.nbas), deriv=0)[0]
        res['ao1'] = ev.eval(aopts - origin, np.arange(mol.nbas), deriv=1)
        np.savez_compressed(os.path.join(HERE, 'int3c1e_%s.npz' % tag), **res)

    # -- a K build on a small grid (reference math: dense A contracted) ------
    from pyscf_wb97mv_fast_gb300.grids import build_grids
    mol = Molecule.build(water_dimer(), 'synthetic-svp')
    g = build_grids(mol, level=0)
    rng = np.random.default_rng(5)
    sel = np.sort(rng.choice(g.size, 160, replace=False))
    coords, weights = g.coords[sel], g.weights[sel]
    rm = RefMol(mol)
    pairs = rsp.ShellPairs(rm)
    origin = mol.atom_coords().mean(axis=0)
    ev = rao.AoEvaluator(rm, np, pack=rao.ShellPack(rm, origin=origin),
                         mem_budget=1 << 28, dtype='float64', verify=False)
    X = ev.eval(coords - origin, np.arange(mol.nbas), deriv=0)[0]
    c = rng.normal(size=(mol.nao, 10))
    c, _ = np.linalg.qr(c)
    dm = 2.0 * c @ c.T
    res = {'coords': coords, 'weights': weights, 'dm': dm}
    for omega in (0.0, 0.3):
        A = rsp.int3c1e_reference(pairs, coords, omega=omega)
        F = X @ dm
        G = np.einsum('gmn,gm->gn', A, F)
        K = X.T @ (weights[:, None] * G)
        res['K_w%g' % omega] = (K + K.T) * 0.5
    np.savez_compressed(os.path.join(HERE, 'k_svp.npz'), **res)

    # -- VV10 kernel sum (reference NumPy path, Kahan tiles) ------------------
    rng = np.random.default_rng(9)
    n = 700
    xyz = np.concatenate([rng.uniform(-4, 4, (n - 200, 3)),
                          rng.uniform(-4, 4, (200, 3)) + [30.0, 0.0, 0.0]])
    q = rng.uniform(1e-4, 1e-2, n)
    w0 = rng.uniform(0.3, 3.0, n)
    kap = rng.uniform(0.4, 2.0, n)
    kern = rvv.Vv10Kernel(np, mem_budget=1 << 24, tile_tol=0.0, outer_chunk=128)
    F, U, W = kern.kernel_sum(xyz.astype(np.float32), q, w0, kap)
    np.savez_compressed(os.path.join(HERE, 'vv10.npz'), xyz=xyz, q=q, w0=w0,
                        kappa=kap, F=F, U=U, W=W)
    # -- the VV10 flow (gpu_nr_nlc_vxc, NumPy backend, FP64 AO and GEMMs) -------
    mol = Molecule.build(water_dimer(), 'synthetic-svp')
    rm = RefMol(mol)
    g = build_grids(mol, level=0)
    rng = np.random.default_rng(13)
    sel = np.sort(rng.choice(g.size, 1500, replace=False))
    origin = mol.atom_coords().mean(axis=0)
    ev = rao.AoEvaluator(rm, np, pack=rao.ShellPack(rm, origin=origin),
                         mem_budget=1 << 28, dtype='float64', verify=False)
    ctx = types.SimpleNamespace(
        xp=np, blksize=560, origin=origin, evaluator=ev, gemm_dtype='float64',
        kernel=rvv.Vv10Kernel(np, mem_budget=1 << 24, tile_tol=0.0))
    grids = types.SimpleNamespace(coords=g.coords[sel], weights=g.weights[sel],
                                  non0tab=None, mol=None)
    ni = types.SimpleNamespace(nlc_coeff=lambda xc: [((6.0, 0.01), 1.0)])
    c = np.zeros((mol.nao, 10))
    q, _ = np.linalg.qr(rng.normal(size=(mol.nao, 10)))
    dm = 2.0 * q @ q.T
    nelec, exc, vmat = rvv.gpu_nr_nlc_vxc(ctx, ni, rm, grids, 'wb97m-v', dm)
    np.savez_compressed(os.path.join(HERE, 'vv10_flow.npz'), coords=grids.coords,
                        weights=grids.weights, dm=dm, nelec=nelec, exc=exc,
                        vmat=vmat, nlc_b=6.0, nlc_c=0.01)
    print('golden fixtures written to', HERE)


if __name__ == '__main__':
    main()
