import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line('markers', 'gpu: needs a CUDA GPU (sm_103a) and the '
                            'native library; skipped when no GPU is visible')
    config.addinivalue_line('markers', 'slow: long-running; skipped unless '
                            '--slow is given')


def pytest_addoption(parser):
    parser.addoption('--slow', action='store_true', default=False,
                     help='also run tests marked slow')


def _gpu_available():
    try:
        import torch
        return torch.cuda.is_available() and torch.cuda.device_count() > 0
    except Exception:                      # noqa: BLE001
        return False


def pytest_collection_modifyitems(config, items):
    gpu_ok = None
    skip_gpu = pytest.mark.skip(reason='no CUDA GPU visible')
    skip_slow = pytest.mark.skip(reason='slow; use --slow')
    run_slow = config.getoption('--slow')
    for item in items:
        if item.get_closest_marker('slow') and not run_slow:
            item.add_marker(skip_slow)
        if item.get_closest_marker('gpu'):
            if gpu_ok is None:
                gpu_ok = _gpu_available()
            if not gpu_ok:
                item.add_marker(skip_gpu)


@pytest.fixture(scope='session', autouse=True)
def native_built():
    """The native library and the oracle are compiled once per session
    (no-ops when they are up to date)."""
    from pyscf_wb97mv_fast_gb300 import build
    build.build()
    import oracle
    oracle.build()
