"""The allocation-free VV10 entry point, wb_vv10_kernel_sum_noalloc.

It exists for callers that cannot let the library allocate device memory:
for example a host framework that reserves all GPU memory up front and
hands out fixed arenas, where a cudaMalloc during a request could fail or
stall the device.  Its scratch is a fixed-size device array inside the
library.  This file checks, through the C ABI, that two calls in a row give
the results of the allocating entry point wb_vv10_kernel_sum, and that a
size above the array's limit is rejected with a clear error.

The file is named to be collected last, so that a run stopping at the
first failure has run every other test before it.
"""
import ctypes

import numpy as np
import pytest

from pyscf_wb97mv_fast_gb300 import _native

pytestmark = pytest.mark.gpu


def _inputs(n, seed):
    import torch
    rng = np.random.default_rng(seed)
    dev = 'cuda'
    return (torch.as_tensor(rng.uniform(-6, 6, (n, 3)), dtype=torch.float32, device=dev),
            torch.as_tensor(rng.uniform(1e-4, 1e-2, n), dtype=torch.float32, device=dev),
            torch.as_tensor(rng.uniform(0.3, 3.0, n), dtype=torch.float32, device=dev),
            torch.as_tensor(rng.uniform(0.4, 2.0, n), dtype=torch.float32, device=dev))


def _call(name, args, n, tile_tol):
    import torch
    lib = _native.lib()
    out = [torch.full((n,), np.nan, dtype=torch.float64, device='cuda')
           for _ in range(3)]
    kept = ctypes.c_int64(-1)
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    st = getattr(lib, name)(*[_native.ptr(a) for a in args], n, tile_tol,
                            *[_native.ptr(o) for o in out], stream,
                            ctypes.byref(kept))
    _native.check(st, name)
    torch.cuda.synchronize()
    return [o.cpu().numpy() for o in out], kept.value


@pytest.mark.parametrize('n,tile_tol', [(3000, 0.0), (2600, 1e-9)])
def test_noalloc_matches_allocating_entry_twice(n, tile_tol):
    args = _inputs(n, 7)
    ref, kept_ref = _call('wb_vv10_kernel_sum', args, n, tile_tol)
    for _ in range(2):                       # the shared array is reused
        got, kept = _call('wb_vv10_kernel_sum_noalloc', args, n, tile_tol)
        assert kept == kept_ref
        for g, r in zip(got, ref):
            assert np.all(np.isfinite(g))
            # same kernels, same summation order: bitwise equal
            np.testing.assert_array_equal(g, r)


def test_noalloc_second_input_does_not_see_the_first():
    """The counter restarts and the tile statistics are rewritten per call:
    a different (smaller) input right after a larger one still matches."""
    big = _inputs(5000, 1)
    small = _inputs(700, 2)
    _call('wb_vv10_kernel_sum_noalloc', big, 5000, 0.0)
    ref, kref = _call('wb_vv10_kernel_sum', small, 700, 0.0)
    got, k = _call('wb_vv10_kernel_sum_noalloc', small, 700, 0.0)
    assert k == kref == 700 * 700
    for g, r in zip(got, ref):
        np.testing.assert_array_equal(g, r)


def test_noalloc_rejects_sizes_above_its_scratch():
    import torch
    n = _native.WB_VV10_NOALLOC_MAX_POINTS + 1
    lib = _native.lib()
    dummy = torch.zeros(4, dtype=torch.float32, device='cuda')
    out = torch.zeros(4, dtype=torch.float64, device='cuda')
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    st = lib.wb_vv10_kernel_sum_noalloc(*[_native.ptr(dummy)] * 4, n, 0.0,
                                        *[_native.ptr(out)] * 3, stream, None)
    assert st == _native.WB_ERR_INVALID_ARGUMENT
    assert b'WB_VV10_NOALLOC_MAX_POINTS' in lib.wb_last_error()
