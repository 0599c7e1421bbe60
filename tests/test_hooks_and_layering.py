"""Hook mechanics, the install boundary with stand-in PySCF modules, and
package layering (CPU)."""
import subprocess
import sys
import types

import numpy as np
import pytest

from pyscf_wb97mv_fast_gb300.core.hooks import HookSet, reset_diis, track_residual


class Base:
    def method(self):
        return 'base'


def test_wrap_restores_module_function_and_instance_shadow():
    mod = types.ModuleType('m')
    mod.f = lambda x: x + 1
    orig = mod.f
    obj = Base()
    with HookSet() as hooks:
        hooks.wrap(mod, 'f', lambda o: (lambda x: o(x) * 10))
        hooks.wrap(obj, 'method', lambda o: (lambda: 'hooked:' + o()))
        assert mod.f(1) == 20
        assert obj.method() == 'hooked:base'
        assert 'method' in obj.__dict__
    assert mod.f is orig
    assert 'method' not in obj.__dict__ and obj.method() == 'base'


def test_restore_order_and_closed_state():
    calls = []
    hooks = HookSet()
    mod = types.ModuleType('m')
    mod.v = 1
    hooks.on_restore(lambda: calls.append('first'))
    hooks.wrap(mod, 'v', lambda o: o + 1)
    hooks.on_restore(lambda: calls.append(('last', mod.v)))
    hooks.restore_all()
    assert calls == [('last', 2), 'first'] and mod.v == 1
    with pytest.raises(RuntimeError):
        hooks.wrap(mod, 'v', lambda o: o)
    with pytest.raises(RuntimeError):
        hooks.on_restore(lambda: None)


def test_reset_diis_and_track_residual():
    class FakeDiis:
        space = 8
        _buffer = {'x': 1}
        _bookkeep = [1, 2]
        _head = 2
        _H = object()
        _xprev = object()
    d = FakeDiis()
    d._buffer = {'x': 1}
    reset_diis(d)
    assert d._buffer == {} and d._bookkeep == [] and d._head == 0
    assert d._H is None and d.space == 8
    reset_diis(None)

    class Mf:
        callback = None
    mf = Mf()
    seen = []
    with HookSet() as hooks:
        track_residual(hooks, mf, seen.append)
        mf.callback({'norm_gorb': 3.5})
    assert seen == [3.5] and mf.callback is None


def _fake_mf():
    class Sgx:
        pass
    df = Sgx()
    df._rsh_df = {'0.300000': Sgx()}
    mf = types.SimpleNamespace(with_df=df, mol=None, _numint=types.SimpleNamespace())
    return mf, Sgx


def test_install_routes_only_this_mf_and_restores():
    from pyscf_wb97mv_fast_gb300.gpu.install import install_gpu
    mf, Sgx = _fake_mf()
    mod = types.ModuleType('fake_sgx_jk')
    calls = []
    mod.get_k_only = lambda sgx, dm, hermi=1, tol=1e-13: calls.append(sgx) or 'cpu'
    orig = mod.get_k_only
    hooks = install_gpu(mf, k=True, vv10=False, semilocal=False,
                        sgx_jk_module=mod)
    assert mod.get_k_only is not orig
    other = Sgx()
    assert mod.get_k_only(other, None) == 'cpu'   # foreign SGX object: original
    assert calls == [other]
    hooks.restore_all()
    assert mod.get_k_only is orig


def test_install_semilocal_hook_wraps_and_restores_nr_rks():
    from pyscf_wb97mv_fast_gb300.gpu.install import install_gpu
    mf, _ = _fake_mf()
    stock = lambda *a, **k: 'cpu'
    mf._numint.nr_rks = stock
    hooks = install_gpu(mf, semilocal=True, k=False, vv10=False,
                        functional_factory=lambda xc, ni: None)
    assert mf._numint.nr_rks is not stock
    assert mf._numint.nr_rks.__name__ == 'nr_rks'
    hooks.restore_all()
    assert mf._numint.nr_rks is stock
    with pytest.raises(ValueError):
        install_gpu(mf, backend='numpy', k=False, vv10=False)
    with pytest.raises(TypeError):
        install_gpu(types.SimpleNamespace(mol=None), semilocal=True, k=False,
                    vv10=False)


def test_oom_retry_halves_tile_then_reraises():
    from pyscf_wb97mv_fast_gb300.gpu.install import _run_with_oom_retry

    class B:
        def __init__(self, blksize):
            self.blksize = blksize

        def with_blksize(self, n):
            return B(n)
    seen = []

    def flow(b):
        seen.append(b.blksize)
        raise MemoryError('out of memory')
    with pytest.raises(MemoryError):
        _run_with_oom_retry(flow, B(1024))
    assert seen == [1024, 512, 256]

    def ok_second(b):
        seen.append(b.blksize)
        if b.blksize > 600:
            raise MemoryError('out of memory')
        return b.blksize
    seen.clear()
    assert _run_with_oom_retry(ok_second, B(1024)) == 512

    def other(b):
        raise ValueError('not an OOM')
    with pytest.raises(ValueError):
        _run_with_oom_retry(other, B(1024))


def test_import_has_no_side_effects():
    code = ('import sys, pyscf_wb97mv_fast_gb300, pyscf_wb97mv_fast_gb300.gpu.install, '
            'pyscf_wb97mv_fast_gb300.gpu.sgx_k, pyscf_wb97mv_fast_gb300.core.sgx_patch, '
            'pyscf_wb97mv_fast_gb300.staging.schedule, pyscf_wb97mv_fast_gb300.gpu.xc;'
            'print(any(m == "pyscf" or m.startswith("pyscf.") for m in sys.modules),'
            ' "torch" in sys.modules)')
    out = subprocess.run([sys.executable, '-c', code], capture_output=True,
                         text=True, check=True).stdout.split()
    assert out == ['False', 'False']


def test_rsh_omegas_from_the_functional():
    from pyscf_wb97mv_fast_gb300.gpu.install import rsh_omegas

    class NumInt:
        def __init__(self, coeff):
            self.coeff = coeff

        def rsh_and_hybrid_coeff(self, xc, spin=0):
            if self.coeff is None:
                raise KeyError(xc)
            return self.coeff

    def mf(coeff):
        return types.SimpleNamespace(_numint=NumInt(coeff), xc='x',
                                     mol=types.SimpleNamespace(spin=0))

    assert rsh_omegas(mf((0.3, 1.0, 0.15))) == (0.0, 0.3)     # wB97M-V
    assert rsh_omegas(mf((0.3, 1.0, 0.0))) == (0.3,)          # LR only
    assert rsh_omegas(mf((0.0, 0.0, 0.25))) is None           # global hybrid
    assert rsh_omegas(mf(None)) is None
    assert rsh_omegas(types.SimpleNamespace()) is None


def test_builder_pending_set_only_matches_same_inputs():
    import numpy as np
    from pyscf_wb97mv_fast_gb300.gpu.sgx_k import GpuKBuilder
    b = GpuKBuilder.__new__(GpuKBuilder)
    dm = np.arange(9.0).reshape(3, 3)
    proj = np.eye(3)
    key = ('grid', False, 1e-11, 'ozaki')
    K = np.ones((3, 3))
    b._pending = (key, dm.copy(), proj.copy(), {0.3: K})
    assert b._take_pending(key, dm, proj, 0.0) is None        # omega miss
    assert b._pending is None                                 # dropped
    b._pending = (key, dm.copy(), proj.copy(), {0.3: K})
    other = dm.copy()
    other[0, 0] += 1.0
    assert b._take_pending(key, other, proj, 0.3) is None     # density miss
    b._pending = (key, dm.copy(), proj.copy(), {0.3: K})
    assert b._take_pending(('g2',) + key[1:], dm, proj, 0.3) is None
    b._pending = (key, dm.copy(), proj.copy(), {0.3: K})
    assert b._take_pending(key, dm, 2 * proj, 0.3) is None    # projector miss
    b._pending = (key, dm.copy(), proj.copy(), {0.3: K})
    assert b._take_pending(key, dm, proj, 0.3) is K           # hit, consumed
    assert b._pending is None


class FakeMole:
    """PySCF Mole accessors over a Molecule (the ones Molecule.from_pyscf
    reads), with switches for the inputs the GPU path refuses."""

    def __init__(self, mol, cart=False, kappa=0, extra_l=None):
        self._m = mol
        self.cart = cart
        self.basis = 'fake'
        self._shells = list(mol.shells)
        if extra_l is not None:
            from pyscf_wb97mv_fast_gb300.basis import Shell
            self._shells.append(Shell(0, extra_l, [1.0], [[1.0]]))
        self._kappa = kappa
        self._bas = np.asarray([[sh.atom, sh.l, sh.nprim, sh.nctr]
                                for sh in self._shells], dtype=np.int32)
        self.natm = mol.natm
        self.nbas = len(self._shells)

    def bas_kappa(self, i):
        return self._kappa

    def bas_angular(self, i):
        return self._shells[i].l

    def bas_exp(self, i):
        return self._shells[i].exps

    def _libcint_ctr_coeff(self, i):
        return self._shells[i].coeffs

    def atom_symbol(self, i):
        return self._m.symbols[i]

    def atom_coords(self):
        return self._m.atom_coords()


def test_from_pyscf_reads_a_mole_back():
    from pyscf_wb97mv_fast_gb300.basis import Molecule
    from pyscf_wb97mv_fast_gb300.systems import water_dimer
    mol = Molecule.build(water_dimer(), 'synthetic-tzvp', gen_contract=True)
    back = Molecule.from_pyscf(FakeMole(mol))
    a, b = mol.packed(), back.packed()
    assert back.nao == mol.nao and set(a) == set(b)
    for key in a:
        assert np.array_equal(a[key], b[key]), key


@pytest.mark.parametrize('bad', ['cart', 'spinor', 'l4', 'not_a_mole'])
def test_install_refuses_out_of_scope_molecules_up_front(bad):
    from pyscf_wb97mv_fast_gb300 import _native
    from pyscf_wb97mv_fast_gb300.basis import Molecule
    from pyscf_wb97mv_fast_gb300.gpu.install import install_gpu
    from pyscf_wb97mv_fast_gb300.systems import water_dimer
    mol = Molecule.build(water_dimer(), 'synthetic-svp')
    fake = {'cart': lambda: FakeMole(mol, cart=True),
            'spinor': lambda: FakeMole(mol, kappa=-1),
            'l4': lambda: FakeMole(mol, extra_l=4),
            'not_a_mole': lambda: object()}[bad]()
    mf, _ = _fake_mf()
    mf.mol = fake
    mod = types.ModuleType('fake_sgx_jk')
    mod.get_k_only = lambda *a: None
    orig = mod.get_k_only
    with pytest.raises(_native.Unsupported):
        install_gpu(mf, k=True, semilocal=False, vv10=False, sgx_jk_module=mod)
    assert mod.get_k_only is orig                  # nothing was hooked
    mf.mol = FakeMole(mol)                         # in scope: installs
    install_gpu(mf, k=True, semilocal=False, vv10=False,
                sgx_jk_module=mod).restore_all()


def test_restore_all_undoes_any_sequence_of_wraps():
    """Random sequences of wraps (the same name several times included) on
    a module function, an instance's own attribute and a class method seen
    through an instance: restore_all leaves every object as it was,
    including which attributes the instance owns."""
    hyp = pytest.importorskip('hypothesis')
    st = pytest.importorskip('hypothesis.strategies')

    class K:
        def meth(self):
            return 'class'

    @hyp.settings(max_examples=60, deadline=None)
    @hyp.given(st.lists(st.sampled_from(['mod.f', 'obj.own', 'obj.meth']),
                        max_size=8))
    def check(seq):
        mod = types.ModuleType('m')
        mod.f = lambda: 'mod'
        obj = K()
        obj.own = lambda: 'own'
        before = (mod.f, dict(vars(obj)))
        hooks = HookSet()
        for i, target in enumerate(seq):
            owner, name = {'mod.f': (mod, 'f'), 'obj.own': (obj, 'own'),
                           'obj.meth': (obj, 'meth')}[target]
            hooks.wrap(owner, name, lambda orig, i=i: (lambda *a: (i, orig)))
        hooks.restore_all()
        assert mod.f is before[0] and vars(obj) == before[1]
        assert obj.meth() == 'class' and obj.own() == 'own'
        with pytest.raises(RuntimeError):
            hooks.wrap(mod, 'f', lambda o: o)

    check()


def test_install_gpu_defaults_are_the_references():
    """The keyword defaults of install_gpu equal the reference's signature
    (pyscf_wb97mv_fast/gpu/install.py:209-213); the additions come after
    them and are opt-in."""
    import inspect
    from pyscf_wb97mv_fast_gb300.gpu.install import install_gpu
    ref = dict(backend=None, blksize=8192, vv10_tile_tol=0.0,
               functional_factory=None, verify_ao=True, gemm_dtype='float32',
               dtype='float32', mem_fraction=0.6, overlap=True, semilocal=True,
               k=False, k_tile_tol=1e-11, openblas_threads=1)
    params = list(inspect.signature(install_gpu).parameters.values())
    assert [p.name for p in params[:len(ref) + 1]] == ['mf'] + list(ref)
    for p in params[1:len(ref) + 1]:
        assert p.default == ref[p.name], p.name
    extra = {p.name: p.default for p in params[len(ref) + 1:]}
    assert extra == dict(vv10=True, k_gemm='ozaki', sgx_jk_module=None,
                         k_omegas='auto', k_precision='fp32')


def test_install_default_places_no_k_hook():
    """install_gpu(mf) with the reference's default k=False leaves the
    module function get_k_only alone."""
    from pyscf_wb97mv_fast_gb300.gpu.install import install_gpu
    mod = types.SimpleNamespace(get_k_only=lambda *a, **k: 'cpu')
    orig = mod.get_k_only
    mf = types.SimpleNamespace(mol=None, with_df=object())
    hooks = install_gpu(mf, semilocal=False, vv10=False, overlap=False,
                        sgx_jk_module=mod, openblas_threads=None)
    assert mod.get_k_only is orig
    hooks.restore_all()


def test_install_rejects_unknown_gemm_dtype():
    from pyscf_wb97mv_fast_gb300.gpu.install import install_gpu
    mf = types.SimpleNamespace(mol=None)
    with pytest.raises(ValueError):
        install_gpu(mf, semilocal=False, vv10=False, gemm_dtype='bfloat16')


class _FakeBlas:
    def __init__(self, parallel, threads):
        self.par, self.threads, self.calls = parallel, threads, []

    def lib(self):
        from pyscf_wb97mv_fast_gb300.core.blas_threads import BlasLib
        return BlasLib('fake', lambda: self.par, lambda: self.threads,
                       self._set)

    def _set(self, n):
        self.calls.append(n)
        self.threads = n


def test_openblas_limit_touches_pthreads_builds_and_restores():
    from pyscf_wb97mv_fast_gb300.core.blas_threads import limit_openblas_threads
    pth, omp, seq = _FakeBlas(1, 8), _FakeBlas(2, 8), _FakeBlas(0, 1)
    undo = limit_openblas_threads(1, libs=[pth.lib(), omp.lib(), seq.lib()],
                                  environ={})
    assert pth.threads == 1 and omp.calls == [] and seq.calls == []
    undo()
    assert pth.threads == 8


def test_openblas_limit_respects_user_environment():
    from pyscf_wb97mv_fast_gb300.core.blas_threads import limit_openblas_threads
    pth = _FakeBlas(1, 8)
    assert limit_openblas_threads(1, libs=[pth.lib()],
                                  environ={'OPENBLAS_NUM_THREADS': '4'}) is None
    assert pth.calls == []
    assert limit_openblas_threads(1, libs=[_FakeBlas(0, 1).lib()], environ={}) is None


def test_openblas_limit_reads_this_process_maps():
    """The real scan runs (numpy's OpenBLAS, when it is a pthreads build,
    is found and limited, then restored)."""
    from pyscf_wb97mv_fast_gb300.core import blas_threads
    libs = blas_threads.mapped_blas_libraries()
    before = [int(lib.get_threads()) for lib in libs]
    undo = blas_threads.limit_openblas_threads(1, libs=libs, environ={})
    if undo is not None:
        undo()
    assert [int(lib.get_threads()) for lib in libs] == before
