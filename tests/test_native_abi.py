"""The C-ABI library: loads without a GPU, exports every symbol the header
declares, host-side routines, clean errors.  CPU only."""
import ctypes
import os
import re

import numpy as np
import pytest

from pyscf_wb97mv_fast_gb300 import _native

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def header_functions():
    names = set()
    for fn in os.listdir(os.path.join(ROOT, 'include')):
        if fn.endswith('.h'):
            with open(os.path.join(ROOT, 'include', fn)) as fh:
                text = fh.read()
            names.update(re.findall(r'^\s*(?:const\s+)?[A-Za-z_][\w\s\*]*?\b(wb_\w+)\s*\(',
                                    text, flags=re.M))
    return sorted(names)


def test_library_exports_every_header_function():
    lib = _native.lib()
    names = header_functions()
    assert len(names) >= 15
    for name in names:
        assert hasattr(lib, name), name
    assert set(names) <= set(_native.EXPORTED) | {'wb_cosx'}


def header_prototypes():
    """{name: (return type, [parameter declarations])} of every function
    the headers declare (comments stripped)."""
    out = {}
    for fn in os.listdir(os.path.join(ROOT, 'include')):
        if not fn.endswith('.h'):
            continue
        with open(os.path.join(ROOT, 'include', fn)) as fh:
            text = fh.read()
        text = re.sub(r'/\*.*?\*/', ' ', text, flags=re.S)
        text = re.sub(r'//[^\n]*', ' ', text)
        for ret, name, params in re.findall(
                r'([A-Za-z_][\w \t\*]*?)\b(wb_\w+)\s*\(([^()]*)\)\s*;', text):
            plist = [p.strip() for p in params.split(',')]
            if plist == ['void'] or plist == ['']:
                plist = []
            out[name] = (' '.join(ret.split()), plist)
    return out


def _param_kind(decl):
    if '*' in decl or '[' in decl:
        return 'ptr'
    words = [w for w in decl.replace('const', ' ').split()]
    return words[0] if len(words) >= 2 else words[-1]


def test_ctypes_signatures_match_the_header():
    """Every argtypes / restype that the Python side declares has the
    header's arity and, parameter by parameter, its kind (a pointer or the
    same scalar type): a mismatch would hand a kernel a wrong pointer or
    size without any error on the host."""
    lib = _native.lib()
    scalars = {'int': ctypes.c_int, 'int64_t': ctypes.c_int64,
               'double': ctypes.c_double, 'size_t': ctypes.c_size_t}
    rets = {'int': ctypes.c_int, 'int64_t': ctypes.c_int64,
            'size_t': ctypes.c_size_t, 'const char*': ctypes.c_char_p}
    protos = header_prototypes()
    assert set(protos) == set(header_functions())
    for name, (ret, params) in protos.items():
        fn = getattr(lib, name)
        assert fn.restype is rets[ret.replace(' *', '*')], (name, ret)
        assert fn.argtypes is not None, name
        assert len(fn.argtypes) == len(params), (name, params)
        for decl, at in zip(params, fn.argtypes):
            kind = _param_kind(decl)
            if kind == 'ptr':
                assert (at in (ctypes.c_void_p, ctypes.c_char_p)
                        or issubclass(at, ctypes._Pointer)), (name, decl, at)
            else:
                assert at is scalars[kind], (name, decl, at)


def test_status_strings_and_version():
    lib = _native.lib()
    assert lib.wb_version() >= 1
    assert lib.wb_status_string(0) == b'ok'
    assert lib.wb_status_string(2) == b'unsupported input'


def test_host_boys_matches_oracle():
    import oracle
    from pyscf_wb97mv_fast_gb300.cosx import boys_f64_host
    for t in (0.0, 0.01, 2.5, 18.0, 39.9, 40.0, 120.0, 1e5):
        assert np.allclose(boys_f64_host(12, t), oracle.boys(12, t), rtol=1e-13,
                           atol=0)
    with pytest.raises(_native.NativeError):
        boys_f64_host(3, -1.0)


def test_becke_partition_matches_numpy():
    from pyscf_wb97mv_fast_gb300.cosx import becke_partition
    from pyscf_wb97mv_fast_gb300.grids import becke_weights_reference
    rng = np.random.default_rng(3)
    atoms = rng.normal(size=(7, 3)) * 2.0
    pts = rng.normal(size=(300, 3)) * 3.0
    own = rng.integers(0, 7, 300)
    a = becke_partition(pts, own, atoms)
    b = becke_weights_reference(pts, atoms, own)
    assert np.max(np.abs(a - b)) < 1e-13
    with pytest.raises(_native.NativeError):
        becke_partition(pts, np.full(300, 9), atoms)


def test_create_without_device_is_a_clean_error():
    try:
        import torch
        if torch.cuda.is_available():
            pytest.skip('a GPU is present')
    except ImportError:
        pass
    from helpers import dimer
    mol = dimer()
    p = mol.packed()
    b = _native.WbBasis(p['natm'], p['nbas'], _native.ptr(p['atom_coords']),
                        _native.ptr(p['shell_atom']), _native.ptr(p['shell_l']),
                        _native.ptr(p['shell_nprim']), _native.ptr(p['shell_nctr']),
                        _native.ptr(p['shell_exp_off']),
                        _native.ptr(p['shell_coef_off']), _native.ptr(p['exps']),
                        _native.ptr(p['coeffs']))
    origin = np.zeros(3)
    h = ctypes.c_void_p()
    st = _native.lib().wb_cosx_create(ctypes.byref(b), _native.ptr(origin), 1e-14,
                                      ctypes.byref(h))
    assert st == _native.WB_ERR_NO_DEVICE
    assert b'no CUDA device' in _native.lib().wb_last_error()


def test_f_engine_switch_without_a_device():
    """The F-product engine is a process-wide host setting: library by
    default, tc selectable, anything else a clean error."""
    from pyscf_wb97mv_fast_gb300 import cosx
    assert cosx.get_f_engine() == 'library'
    assert cosx.set_f_engine('tc') == 'library'
    assert cosx.get_f_engine() == 'tc'
    assert cosx.set_f_engine('library') == 'tc'
    with pytest.raises(ValueError):
        cosx.set_f_engine('triton')
    assert _native.lib().wb_ozaki_set_f_engine(7) != 0
    assert cosx.get_f_engine() == 'library'
