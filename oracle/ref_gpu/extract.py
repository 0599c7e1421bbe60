"""Writes oracle/_ref/ref_kernels.cuh (the reference's CUDA C strings,
unmodified) and oracle/_ref/ref_pairs_<tag>.npz (the reference's
ShellPairsDevice arrays and screening data for this project's bench
molecules, packed by the reference's own Python).

TEST INFRASTRUCTURE ONLY.  Run from the repository root where a reference
checkout exists:
    python -m oracle.ref_gpu.extract <reference checkout>
PySCF is absent, so the few PySCF names the reference imports are stubbed
(cart2sph by this project's basis.cart2sph, a logger, BLKSIZE); the
kernels and the packing are the reference's code.
"""
import os
import sys
import types

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
OUT = os.path.join(ROOT, 'oracle', '_ref')
sys.path.insert(0, ROOT)


def _stubs(ref_root):
    from pyscf_wb97mv_fast_gb300.basis import cart2sph
    pyscf = types.ModuleType('pyscf')
    gto = types.ModuleType('pyscf.gto')
    mole = types.ModuleType('pyscf.gto.mole')
    mole.cart2sph = cart2sph
    eval_gto = types.ModuleType('pyscf.gto.eval_gto')
    eval_gto.BLKSIZE = 56
    lib = types.ModuleType('pyscf.lib')
    logger = types.ModuleType('pyscf.lib.logger')
    for name in ('debug', 'info', 'note', 'warn', 'timer', 'debug1'):
        setattr(logger, name, lambda *a, **k: None)
    lib.logger = logger
    gto.mole = mole
    gto.eval_gto = eval_gto
    pyscf.gto = gto
    pyscf.lib = lib
    for name, mod in (('pyscf', pyscf), ('pyscf.gto', gto), ('pyscf.gto.mole', mole),
                      ('pyscf.gto.eval_gto', eval_gto), ('pyscf.lib', lib),
                      ('pyscf.lib.logger', logger)):
        sys.modules[name] = mod
    xc = types.ModuleType('pyscf_wb97mv_fast.gpu.xc')

    class Unsupported(Exception):
        pass
    xc.Unsupported = Unsupported
    xc._prepare_dm = lambda dm, hermi: np.asarray(dm)
    sys.modules['pyscf_wb97mv_fast.gpu.xc'] = xc
    sys.path.insert(0, ref_root)


class _RefMol:
    """The Mole accessors the reference's ShellPairs reads, over a Molecule."""

    def __init__(self, mol):
        self.m = mol
        self.cart = False
        self.nbas = mol.nbas
        self._bas = mol._bas
        self.basis = 'synthetic'

    def ao_loc_nr(self):
        return self.m.ao_loc_nr()

    def bas_angular(self, i):
        return self.m.bas_angular(i)

    def bas_kappa(self, i):
        return 0

    def bas_nctr(self, i):
        return self.m.bas_nctr(i)

    def bas_nprim(self, i):
        return self.m.bas_nprim(i)

    def bas_exp(self, i):
        return self.m.shells[i].exps

    def _libcint_ctr_coeff(self, i):
        return self.m.shells[i].coeffs

    def atom_coords(self):
        return self.m.atom_coords()


def write_sources():
    from pyscf_wb97mv_fast.gpu import sgx_k, vv10
    src = ['// Extracted unmodified from the reference (gpu/sgx_k.py _FUSED_SRC,',
           '// _SCREEN_SRC; gpu/vv10.py _FUSED_SRC); build output, not tracked.',
           sgx_k._FUSED_SRC, sgx_k._SCREEN_SRC, vv10._FUSED_SRC]
    os.makedirs(OUT, exist_ok=True)
    with open(os.path.join(OUT, 'ref_kernels.cuh'), 'w') as fh:
        fh.write('\n'.join(src))
    return vv10._FUSED_TILE


def write_pairs(tag, mol, origin):
    from pyscf_wb97mv_fast.gpu.shellpairs import ShellPairs
    from pyscf_wb97mv_fast.gpu import sgx_k
    rm = _RefMol(mol)
    pairs = ShellPairs(rm)
    dev = pairs.to_device(np, origin=origin)
    host = sgx_k._HostPairs(pairs)
    out = {k: np.asarray(getattr(dev, k)) for k in (
        'sh_dims', 'sh_Mc', 'sh_MT', 'sh_Mc_lo', 'sh_MT_lo', 'pair_sh', 'prim_p',
        'prim_prefac', 'prim_prefac_lo', 'prim_P_hi', 'prim_P_lo', 'prim_E')}
    f32 = np.float32
    ao_loc = np.asarray(mol.ao_loc_nr(), dtype=np.int64)
    out.update(
        scr_P=(pairs.prim_P - origin).astype(f32),
        scr_pref=np.nextafter(pairs.prim_bound_pref.astype(f32), f32(np.inf)),
        scr_pp=pairs.prim_pp.astype(f32),
        scr_poff=pairs.prim_offsets.astype(np.int32),
        scr_tau=np.nextafter(pairs.pair_tau.astype(f32), f32(np.inf)),
        scr_ish=pairs.pair_rows[:, 2].astype(np.int32),
        scr_jsh=pairs.pair_rows[:, 3].astype(np.int32),
        pair_class=host.pair_class.astype(np.int32),
        ao_loc=ao_loc.astype(np.int32), origin=np.asarray(origin, dtype=np.float64),
        nao=np.int64(pairs.nao), npairs=np.int64(pairs.npairs))
    # the per-omega constants of the class kernels, by the reference's own
    # GpuKBuilder._omega_data (gpu/sgx_k.py:783-811)
    holder = types.SimpleNamespace(_omega_cache={}, _pairs_host=host, xp=np)
    for omega in (0.0, 0.3):
        tp_hi, tp_lo, cn_hi, cn_lo = sgx_k.GpuKBuilder._omega_data(holder, omega)
        for name, v in (('tp_hi', tp_hi), ('tp_lo', tp_lo), ('cn_hi', cn_hi),
                        ('cn_lo', cn_lo)):
            out['w%g_%s' % (omega, name)] = np.asarray(v)
    np.savez(os.path.join(OUT, 'ref_pairs_%s.npz' % tag), **out)
    return {k: v.nbytes for k, v in out.items()}


# where the build container keeps its read-only reference checkout
DEFAULT_REFERENCE = '/root/reference'


def reference_root(path=None):
    root = path or os.environ.get('WB_REFERENCE_ROOT') or DEFAULT_REFERENCE
    return root if os.path.isdir(os.path.join(root, 'pyscf_wb97mv_fast')) else None


def up_to_date():
    out = [os.path.join(OUT, 'ref_kernels.cuh'),
           os.path.join(OUT, 'ref_pairs_water27_svp.npz')]
    return all(os.path.exists(f) and os.path.getmtime(f) >= os.path.getmtime(__file__)
               for f in out)


def maybe_extract():
    """Extract when a reference checkout is present (the build container)
    and the outputs are missing or older than this script; a no-op on a
    machine without the reference (the outputs then travel with the
    tree).  Runs in a child process: the stubs it installs stay there."""
    if reference_root() is None or up_to_date():
        return False
    import subprocess
    res = subprocess.run([sys.executable, '-m', 'oracle.ref_gpu.extract'], cwd=ROOT,
                         capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError('reference extraction failed:\n' + res.stderr[-2000:])
    return True


def main():
    args = [a for a in sys.argv[1:] if not a.startswith('--')]
    ref_root = reference_root(args[0] if args else None)
    if ref_root is None:
        raise SystemExit('usage: python -m oracle.ref_gpu.extract <reference checkout>')
    _stubs(ref_root)
    write_sources()
    from pyscf_wb97mv_fast_gb300.basis import Molecule
    from pyscf_wb97mv_fast_gb300.systems import water_cluster
    mol = Molecule.build(water_cluster(27, box=10.0, seed=27), 'synthetic-svp')
    origin = mol.atom_coords().mean(axis=0)
    sizes = write_pairs('water27_svp', mol, origin)
    print('ref_pairs_water27_svp: %.1f MB' % (sum(sizes.values()) / 1e6))


if __name__ == '__main__':
    main()
