"""Argument checks of the Python entry points, on the CPU.  The native calls
take raw device pointers and read as many elements as their sizes say, so
a host tensor, another dtype, a wrong shape or a short array must raise a
Python error before any native call.  The engine here is a CosxEngine
without a handle whose device is the CPU, and the native library is a
stand-in that records the calls it gets."""
import numpy as np
import pytest
import torch

from pyscf_wb97mv_fast_gb300 import _native
from pyscf_wb97mv_fast_gb300 import cosx as cosx_mod
from pyscf_wb97mv_fast_gb300.cosx import CosxBatch, CosxEngine, KBuildGraph, round32

NAO = 5


class FakeLib:
    """Stand-in for the native library: sizes are 0 bytes, calls succeed."""

    def __init__(self):
        self.calls = []

    def __getattr__(self, name):
        if name.startswith('wb_'):
            def call(*args):
                if 'workspace_bytes' not in name:
                    self.calls.append(name)
                return 0
            return call
        raise AttributeError(name)


@pytest.fixture
def fake(monkeypatch):
    lib = FakeLib()
    monkeypatch.setattr(_native, 'lib', lambda: lib)
    monkeypatch.setattr(CosxEngine, '_stream', staticmethod(lambda: None))
    eng = object.__new__(CosxEngine)
    eng.nao = NAO
    eng.device = torch.device('cpu')
    eng._h = None
    eng._ws = None
    eng.last_stats = {}
    return eng, lib


def _grid(n=40):
    c = torch.zeros((n, 3), dtype=torch.float64)
    w = torch.ones(n, dtype=torch.float64)
    return c, w


def test_valid_calls_reach_the_native_library(fake):
    eng, lib = fake
    c, w = _grid()
    qd = torch.eye(NAO, dtype=torch.float64)
    eng.get_k_multi(c, w, qd, (0.0, 0.3), stats=False)
    eng.get_k(c, w, qd, 0.3, stats=False)
    eng.get_k_fp64(c, w, qd, (0.0,), stats=False)
    ld = round32(len(w))
    f = torch.zeros((NAO, ld), dtype=torch.float32)
    eng.g(c, w, f, 0.0, stats=False)
    eng.g_multi(c, w, f, (0.0, 0.3), stats=False)
    X = eng.ao_eval(c)
    eng.ozaki_f(X, qd)
    eng.ozaki_k(X, f, w)
    X4 = eng.ao_eval_deriv1(c)
    eng.xc_rho(X4, torch.zeros((4, NAO, ld), dtype=torch.float32), len(w), True)
    eng.xc_aow(X4, torch.zeros((5, ld), dtype=torch.float64), len(w), False)
    assert lib.calls == ['wb_cosx_get_k_multi', 'wb_cosx_get_k', 'wb_cosx_get_k_fp64',
                         'wb_cosx_g', 'wb_cosx_g_multi', 'wb_ao_eval',
                         'wb_cosx_ozaki_f', 'wb_cosx_ozaki_k', 'wb_ao_eval_deriv1',
                         'wb_xc_rho', 'wb_xc_aow']


@pytest.mark.parametrize('case', ['qd_f32', 'qd_shape', 'qd_numpy', 'qd_device',
                                  'w_short', 'w_f32', 'c_shape', 'out_shape',
                                  'out_strided'])
def test_bad_k_arguments_stop_before_the_native_call(fake, case):
    eng, lib = fake
    c, w = _grid()
    qd = torch.eye(NAO, dtype=torch.float64)
    out = None
    if case == 'qd_f32':
        qd = qd.float()
    elif case == 'qd_shape':
        qd = torch.eye(NAO + 1, dtype=torch.float64)
    elif case == 'qd_numpy':
        qd = np.eye(NAO)
    elif case == 'qd_device':
        qd = torch.empty((NAO, NAO), dtype=torch.float64, device='meta')
    elif case == 'w_short':
        w = w[:-1]
    elif case == 'w_f32':
        w = w.float()
    elif case == 'c_shape':
        c = torch.zeros((40, 4), dtype=torch.float64)
    elif case == 'out_shape':
        out = torch.empty((1, NAO, NAO), dtype=torch.float64)
    elif case == 'out_strided':
        out = torch.empty((NAO, 2, NAO), dtype=torch.float64).transpose(0, 1)
    with pytest.raises((TypeError, ValueError)):
        eng.get_k_multi(c, w, qd, (0.0, 0.3), out=out, stats=False)
    assert lib.calls == []


def test_bad_g_ozaki_and_xc_arguments(fake):
    eng, lib = fake
    c, w = _grid()
    ld = round32(len(w))
    with pytest.raises(TypeError):
        eng.g(c, w, torch.zeros((NAO, ld), dtype=torch.float64), 0.0)
    with pytest.raises(ValueError):
        eng.g_multi(c, w, torch.zeros((NAO, ld - 32), dtype=torch.float32), (0.0,))
    X = torch.zeros((NAO, ld), dtype=torch.float64)
    G = torch.zeros((NAO, ld), dtype=torch.float32)
    with pytest.raises(ValueError):
        eng.ozaki_k(X, G, torch.ones(ld + 1, dtype=torch.float64))
    with pytest.raises(ValueError):
        eng.ozaki_k(X, G[:, :32].contiguous(), w)
    with pytest.raises(TypeError):
        eng.ozaki_f(X.float(), torch.eye(NAO, dtype=torch.float64))
    X4 = torch.zeros((4, NAO, ld), dtype=torch.float64)
    with pytest.raises(ValueError):          # MGGA needs four T planes
        eng.xc_rho(X4, torch.zeros((1, NAO, ld), dtype=torch.float32), len(w), True)
    with pytest.raises(ValueError):
        eng.xc_aow(X4, torch.zeros((5, ld), dtype=torch.float64), ld + 1, False)
    with pytest.raises(ValueError):
        eng.ao_eval(c, out=torch.empty((NAO, ld + 32), dtype=torch.float64))
    assert lib.calls == []


def test_batch_run_and_graph_run_check_their_buffers(fake):
    eng, lib = fake
    b = object.__new__(CosxBatch)
    b.engines = [eng]
    b.omegas = (0.0, 0.3)
    b.device = eng.device
    b._b = None
    b.last_stats = {}
    qd = torch.eye(NAO, dtype=torch.float64)
    with pytest.raises(TypeError):
        b.run([qd.float()])
    with pytest.raises(ValueError):
        b.run([qd], out=[torch.empty((1, NAO, NAO), dtype=torch.float64)])
    with pytest.raises(ValueError):
        b.run([qd], out=[])
    b.run([qd])
    assert lib.calls == ['wb_cosx_batch_run']
    g = object.__new__(KBuildGraph)
    g.qd = torch.zeros((NAO, NAO), dtype=torch.float64)
    with pytest.raises(ValueError):
        g.run(np.zeros(NAO))                 # would broadcast into qd


def test_device_arg_messages():
    t = torch.zeros((3, 2), dtype=torch.float64)
    assert cosx_mod.device_arg(t, 't', torch.float64, t.device, (None, 2)) is t
    with pytest.raises(ValueError, match=r'\(\*, 3\)'):
        cosx_mod.device_arg(t, 't', torch.float64, t.device, (None, 3))
    with pytest.raises(TypeError, match='float32'):
        cosx_mod.device_arg(t, 't', torch.float32, t.device)
    with pytest.raises(ValueError, match='contiguous'):
        cosx_mod.device_out(t.T, 't', torch.float64, t.device, (2, 3))


def test_vv10_inputs_must_be_device_tensors_of_one_length():
    from pyscf_wb97mv_fast_gb300.gpu import vv10
    with pytest.raises(ValueError, match='CUDA'):
        vv10.Vv10Kernel().kernel_sum(torch.zeros((4, 3)), np.ones(4), np.ones(4),
                                     np.ones(4))
    with pytest.raises(ValueError, match='CUDA'):
        vv10.Vv10Kernel().kernel_sum_batch([torch.zeros((4, 3))], [np.ones(4)],
                                           [np.ones(4)], [np.ones(4)])
    with pytest.raises(ValueError, match='per molecule'):
        vv10.Vv10Kernel().kernel_sum_batch([], [], [], [])
    with pytest.raises(ValueError, match=r'\(4,\)'):
        vv10._per_point(np.ones(3), 4, torch.device('cpu'), 'q')
