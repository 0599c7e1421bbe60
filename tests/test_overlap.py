"""install_gpu(overlap=True): mf.get_veff runs the XC and VV10 flows on a
worker thread while the stock get_veff builds J and K (the reference's
gpu/install.py:138-206, tested there by tests/gpu/test_install.py:222).
CPU only, on a stand-in DFT object whose stock get_veff follows the sums of
PySCF's rks.get_veff: vxc + vj - vk/2, exc - <dm|vk>/4, ecoul = <dm|vj>/2,
the result tagged with ecoul, exc, vj and vk."""
import threading
import types

import numpy as np
import pytest

from pyscf_wb97mv_fast_gb300.gpu.install import install_gpu, retag

NAO = 6


class Tagged(np.ndarray):
    """Stands in for PySCF's tag_array type: an array with attributes."""


def tag(arr, **tags):
    out = np.asarray(arr).view(Tagged)
    out.__dict__.update(tags)
    return out


class NumInt:
    """nr_rks / nr_nlc_vxc on the class, as PySCF's NumInt has them."""

    def __init__(self, gate=None, fail=False):
        self.libxc = types.SimpleNamespace(is_nlc=lambda xc: True)
        self.gate = gate            # (worker started, J/K started) events
        self.fail = fail
        self.threads = []

    def nr_rks(self, mol, grids, xc, dm, *args, **kwargs):
        self.threads.append(threading.current_thread().name)
        if self.gate is not None:
            self.gate[0].set()
            assert self.gate[1].wait(10), 'J/K never ran beside the XC flow'
        if self.fail:
            raise RuntimeError('xc flow failed')
        return 3.0, -1.25 * np.trace(dm), 0.1 * dm + 0.01

    def nr_nlc_vxc(self, mol, grids, xc, dm, *args, **kwargs):
        return 0.0, 0.02 * np.trace(dm), 0.003 * dm


class Mf:
    def __init__(self, ni):
        self.mol = 'mol'
        self.xc = 'wb97m-v'
        self.nlc = ''
        self._numint = ni
        self.grids = types.SimpleNamespace(coords=np.zeros((4, 3)))
        self.nlcgrids = types.SimpleNamespace(coords=np.zeros((4, 3)))
        self.jk_threads = []

    def do_nlc(self):
        return True

    def initialize_grids(self, mol, dm):
        self.grids.coords = np.zeros((4, 3))

    def get_veff(self, mol=None, dm=None, dm_last=None, vhf_last=None, hermi=1):
        ni = self._numint
        dm = np.asarray(dm)
        self.jk_threads.append(threading.current_thread().name)
        if ni.gate is not None:
            assert ni.gate[0].wait(10), 'the XC flow never started'
            ni.gate[1].set()
        _, exc, vxc = ni.nr_rks(mol, self.grids, self.xc, dm)
        _, enlc, vnlc = ni.nr_nlc_vxc(mol, self.nlcgrids, self.xc, dm)
        exc += enlc
        vxc = vxc + vnlc
        vj, vk = 2.0 * dm, 0.5 * dm @ dm
        vxc = vxc + vj - 0.5 * vk
        exc -= 0.25 * np.einsum('ij,ji->', dm, vk)
        ecoul = 0.5 * np.einsum('ij,ji->', dm, vj)
        return tag(vxc, ecoul=ecoul, exc=exc, vj=vj, vk=vk)


def _dm(seed=0):
    c = np.random.default_rng(seed).normal(size=(NAO, 3))
    return c @ c.T


def _install(mf):
    return install_gpu(mf, k=False, semilocal=False, vv10=False, overlap=True)


def test_overlapped_get_veff_equals_the_serial_one():
    dm = _dm()
    serial = Mf(NumInt()).get_veff('mol', dm)
    ni = NumInt(gate=(threading.Event(), threading.Event()))
    mf = Mf(ni)
    hooks = _install(mf)
    assert 'get_veff' in vars(mf)
    v = mf.get_veff('mol', dm)
    assert np.allclose(v, serial, rtol=0, atol=1e-14)
    for t in ('exc', 'ecoul'):
        assert getattr(v, t) == pytest.approx(getattr(serial, t), abs=1e-13)
    for t in ('vj', 'vk'):
        assert np.array_equal(getattr(v, t), getattr(serial, t))
    # XC on the worker, J/K on this thread, at the same time (the gate)
    assert ni.threads[0] == 'wb-xc' and mf.jk_threads == [threading.current_thread().name]
    (t,) = hooks.timings
    assert set(t) == {'jk', 'xc', 'wait'} and min(t.values()) >= 0.0
    # nr_rks / nr_nlc_vxc are the class's again, not instance attributes
    assert 'nr_rks' not in vars(ni) and 'nr_nlc_vxc' not in vars(ni)
    hooks.restore_all()
    assert 'get_veff' not in vars(mf)


def test_worker_error_is_raised_and_hooks_stay_intact():
    ni = NumInt(fail=True)
    mf = Mf(ni)
    own = lambda *a, **k: (0, 0.0, np.zeros((NAO, NAO)))     # noqa: E731
    ni.nr_nlc_vxc = own                     # an instance attribute (a hook)
    hooks = _install(mf)
    with pytest.raises(RuntimeError, match='xc flow failed'):
        mf.get_veff('mol', _dm(1))
    assert ni.nr_nlc_vxc is own and 'nr_rks' not in vars(ni)
    assert len(hooks.timings) == 1
    hooks.restore_all()


def test_inputs_the_flows_do_not_take_go_to_the_stock_get_veff():
    ni = NumInt()
    mf = Mf(ni)
    hooks = _install(mf)
    dm = _dm(2)
    v = mf.get_veff('mol', dm, hermi=2)
    assert np.array_equal(v, Mf(NumInt()).get_veff('mol', dm))
    mf.get_veff('mol', dm.tolist())         # not an ndarray: stock path
    assert hooks.timings == [] and ni.threads == ['MainThread'] * 2
    hooks.restore_all()


def test_grids_are_set_up_first_and_plain_objects_are_not_wrapped():
    mf = Mf(NumInt())
    mf.grids.coords = None
    hooks = _install(mf)
    mf.get_veff('mol', _dm(3))
    assert mf.grids.coords is not None
    hooks.restore_all()
    plain = types.SimpleNamespace(mol=None, _numint=NumInt())
    hooks = install_gpu(plain, k=False, semilocal=False, vv10=False, overlap=True)
    assert not hasattr(plain, 'get_veff')
    hooks.restore_all()


def test_retag_keeps_the_tags_and_replaces_some():
    a = tag(np.ones((2, 2)), ecoul=1.0, exc=2.0, vj=np.eye(2), vk=None)
    b = retag(a, np.zeros((2, 2)), exc=5.0)
    assert isinstance(b, Tagged) and b.ecoul == 1.0 and b.exc == 5.0
    assert np.array_equal(b.vj, np.eye(2)) and b.vk is None
    assert np.array_equal(b, np.zeros((2, 2)))
