"""ctypes binding of libwb97mv_gb300.so (the C ABI of include/wb97mv_gb300.h).

The library is loaded on first use from pyscf_wb97mv_fast_gb300/_lib/.  If
it is missing the call raises ``NativeLibraryMissing`` -- there is no
Python or CPU fallback for any device entry point.  Status codes become
exceptions: WB_ERR_UNSUPPORTED -> ``Unsupported`` (the reference's
gpu/xc.py:30 exception name), WB_ERR_OUT_OF_MEMORY -> ``DeviceOutOfMemory``
(a MemoryError), the rest -> ``NativeError``.
"""
import ctypes
import os
import threading

from pyscf_wb97mv_fast_gb300 import build as _build

WB_OK = 0
WB_ERR_INVALID_ARGUMENT = 1
WB_ERR_UNSUPPORTED = 2
WB_ERR_CUDA = 3
WB_ERR_CUBLAS = 4
WB_ERR_OUT_OF_MEMORY = 5
WB_ERR_WORKSPACE = 6
WB_ERR_NO_DEVICE = 7

WB_VV10_NOALLOC_MAX_POINTS = 1048576

WB_K_GEMM_NATIVE_FP64 = 0
WB_K_GEMM_EMULATED_FP64 = 1
WB_K_GEMM_OZAKI_BF16 = 2
WB_K_PROFILE = 4
GEMM_MODES = {'native': WB_K_GEMM_NATIVE_FP64,
              'emulated': WB_K_GEMM_EMULATED_FP64,
              'ozaki': WB_K_GEMM_OZAKI_BF16}
PHASES = ('ao', 'f_gemm', 'f_cast', 'g', 'weight_g', 'k_gemm')

NCLASS = 10

EXPORTED = ('wb_cosx_create', 'wb_cosx_destroy', 'wb_cosx_get_info',
            'wb_cosx_export_pairs', 'wb_cosx_workspace_bytes',
            'wb_cosx_get_k', 'wb_cosx_get_k_multi', 'wb_cosx_g',
            'wb_cosx_g_multi', 'wb_cosx_screen_mask', 'wb_scf_int1e',
            'wb_hartree_workspace_bytes', 'wb_hartree', 'wb_ao_eval',
            'wb_ao_eval_deriv1', 'wb_xc_rho', 'wb_xc_aow',
            'wb_int3c1e_dense',
            'wb_boys_fp32', 'wb_boys_f64_host', 'wb_model_flops_per_point',
            'wb_vv10_kernel_sum',
            'wb_becke_partition', 'wb_fp32_fma_probe', 'wb_fp32x2_fma_probe',
            'wb_ozaki_workspace_bytes', 'wb_cosx_ozaki_f', 'wb_cosx_ozaki_k',
            'wb_ozaki_set_f_engine', 'wb_ozaki_get_f_engine',
            'wb_cosx_ozaki_f64', 'wb_cosx_ozaki_k64',
            'wb_vv10_kernel_sum_noalloc', 'wb_vv10_kernel_sum_batch',
            'wb_cosx_fp64_workspace_bytes', 'wb_cosx_get_k_fp64',
            'wb_cosx_set_class_variant', 'wb_cosx_get_class_variant',
            'wb_cosx_k_grad_workspace_bytes', 'wb_cosx_k_grad',
            'wb_cosx_batch_workspace_bytes', 'wb_cosx_batch_create',
            'wb_cosx_batch_run', 'wb_cosx_batch_destroy',
            'wb_status_string',
            'wb_last_error', 'wb_version')


class NativeError(RuntimeError):
    """A failed C-ABI call (status code in .status)."""

    def __init__(self, status, message):
        super().__init__('%s (status %d)' % (message, status))
        self.status = status


class Unsupported(NativeError):
    """Input outside the supported scope (l > 3, caps exceeded, ...)."""


class DeviceOutOfMemory(NativeError, MemoryError):
    """Device allocation failed."""


class NativeLibraryMissing(ImportError):
    """libwb97mv_gb300.so is not built."""


class WbBasis(ctypes.Structure):
    _fields_ = [('natm', ctypes.c_int), ('nbas', ctypes.c_int),
                ('atom_coords', ctypes.c_void_p),
                ('shell_atom', ctypes.c_void_p), ('shell_l', ctypes.c_void_p),
                ('shell_nprim', ctypes.c_void_p),
                ('shell_nctr', ctypes.c_void_p),
                ('shell_exp_off', ctypes.c_void_p),
                ('shell_coef_off', ctypes.c_void_p),
                ('exps', ctypes.c_void_p), ('coeffs', ctypes.c_void_p)]


class WbCosxStats(ctypes.Structure):
    _fields_ = [('tasks_total', ctypes.c_int64), ('tasks_kept', ctypes.c_int64),
                ('integrals', ctypes.c_double), ('model_flops', ctypes.c_double),
                ('tasks_kept_class', ctypes.c_int64 * NCLASS),
                ('model_flops_class', ctypes.c_double * NCLASS),
                ('kernel_launches', ctypes.c_int32), ('reserved', ctypes.c_int32),
                ('phase_ms', ctypes.c_double * 6)]

    def as_dict(self):
        return {'pairs_total': int(self.tasks_total),
                'pairs_kept': int(self.tasks_kept),
                'integrals': float(self.integrals),
                'model_flops': float(self.model_flops),
                'kept_class': [int(x) for x in self.tasks_kept_class],
                'flops_class': [float(x) for x in self.model_flops_class],
                'kernel_launches': int(self.kernel_launches),
                'phase_ms': dict(zip(PHASES, [float(x) for x in self.phase_ms]))}


class WbCosxInfo(ctypes.Structure):
    _fields_ = [('nao', ctypes.c_int), ('nbas', ctypes.c_int),
                ('npairs', ctypes.c_int), ('nprim_pairs', ctypes.c_int),
                ('class_pairs', ctypes.c_int * NCLASS),
                ('class_prim_pairs', ctypes.c_int * NCLASS)]


_LIB = None
_LOCK = threading.Lock()

_P = ctypes.c_void_p
_I64 = ctypes.c_int64
_D = ctypes.c_double
_INT = ctypes.c_int


def _declare(lib):
    sig = {
        'wb_cosx_create': (_INT, [ctypes.POINTER(WbBasis), _P, _D, ctypes.POINTER(_P)]),
        'wb_cosx_destroy': (_INT, [_P]),
        'wb_cosx_get_info': (_INT, [_P, ctypes.POINTER(WbCosxInfo)]),
        'wb_cosx_export_pairs': (_I64, [_P, _P, _I64]),
        'wb_cosx_workspace_bytes': (ctypes.c_size_t, [_P, _I64, _I64]),
        'wb_cosx_get_k': (_INT, [_P, _P, _P, _I64, _P, _D, _D, _I64, _INT, _P,
                                 _P, ctypes.c_size_t, _P,
                                 ctypes.POINTER(WbCosxStats)]),
        'wb_cosx_get_k_multi': (_INT, [_P, _P, _P, _I64, _P, _INT, _P, _D, _I64,
                                       _INT, _P, _P, ctypes.c_size_t, _P,
                                       ctypes.POINTER(WbCosxStats)]),
        'wb_cosx_g': (_INT, [_P, _P, _P, _I64, _P, _D, _D, _P, _P,
                             ctypes.c_size_t, _P, ctypes.POINTER(WbCosxStats)]),
        'wb_cosx_g_multi': (_INT, [_P, _P, _P, _I64, _P, _INT, _P, _D, _P, _P,
                                   ctypes.c_size_t, _P,
                                   ctypes.POINTER(WbCosxStats)]),
        'wb_cosx_screen_mask': (_INT, [_P, _P, _P, _I64, _P, _D, _INT, _P, _P,
                                       ctypes.c_size_t, _P]),
        'wb_scf_int1e': (_INT, [_P, _INT, _P, _P, _P, _P, _P, _P]),
        'wb_hartree_workspace_bytes': (ctypes.c_size_t, [_P, _I64]),
        'wb_hartree': (_INT, [_P, _P, _I64, _P, _D, _INT, _P, _P, ctypes.c_size_t,
                              _P, ctypes.POINTER(ctypes.c_int64)]),
        'wb_ao_eval': (_INT, [_P, _P, _I64, _P, _P]),
        'wb_ao_eval_deriv1': (_INT, [_P, _P, _I64, _P, _P]),
        'wb_xc_rho': (_INT, [_P, _P, _P, _I64, _I64, _INT, _P, _P]),
        'wb_xc_aow': (_INT, [_P, _P, _P, _I64, _I64, _INT, _P, _P]),
        'wb_int3c1e_dense': (_INT, [_P, _P, _I64, _D, _P, _P]),
        'wb_boys_fp32': (_INT, [_P, _I64, _INT, _P, _P]),
        'wb_boys_f64_host': (_INT, [_INT, _D, _P]),
        'wb_model_flops_per_point': (_INT, [_P, _D, _P, _P]),
        'wb_vv10_kernel_sum': (_INT, [_P, _P, _P, _P, _I64, _D, _P, _P, _P, _P,
                                      ctypes.POINTER(_I64)]),
        'wb_becke_partition': (_INT, [_P, _I64, _P, _P, _INT, _P]),
        'wb_vv10_kernel_sum_noalloc': (_INT, [_P, _P, _P, _P, _I64, _D, _P, _P,
                                              _P, _P, ctypes.POINTER(_I64)]),
        'wb_vv10_kernel_sum_batch': (_INT, [_INT, _P, _P, _P, _P, _P, _D, _P, _P, _P,
                                            _P, ctypes.POINTER(_I64)]),
        'wb_fp32_fma_probe': (_INT, [_I64, _P, _I64, _P, ctypes.POINTER(_D)]),
        'wb_fp32x2_fma_probe': (_INT, [_I64, _P, _I64, _P, ctypes.POINTER(_D)]),
        'wb_ozaki_workspace_bytes': (ctypes.c_size_t, [_INT, _I64]),
        'wb_cosx_ozaki_f': (_INT, [_P, _P, _P, _I64, _P, _P, ctypes.c_size_t, _P]),
        'wb_ozaki_set_f_engine': (_INT, [_INT]),
        'wb_cosx_ozaki_f64': (_INT, [_P, _P, _P, _I64, _P, _P, ctypes.c_size_t, _P]),
        'wb_ozaki_get_f_engine': (_INT, []),
        'wb_cosx_ozaki_k': (_INT, [_P, _P, _P, _P, _I64, _INT, _P, _P,
                                   ctypes.c_size_t, _P]),
        'wb_cosx_ozaki_k64': (_INT, [_P, _P, _P, _P, _I64, _INT, _P, _P,
                                     ctypes.c_size_t, _P]),
        'wb_cosx_fp64_workspace_bytes': (ctypes.c_size_t, [_P, _I64]),
        'wb_cosx_set_class_variant': (_INT, [_P, _INT, _INT, _INT]),
        'wb_cosx_k_grad_workspace_bytes': (ctypes.c_size_t, [_P, _I64, _INT]),
        'wb_cosx_k_grad': (_INT, [_P, _P, _P, _I64, _P, _D, _D, _INT, _P, _P,
                                  ctypes.c_size_t, _P]),
        'wb_cosx_get_class_variant': (_INT, [_P, _INT, ctypes.POINTER(_INT),
                                             ctypes.POINTER(_INT)]),
        'wb_cosx_get_k_fp64': (_INT, [_P, _P, _P, _I64, _P, _INT, _P, _D, _P, _P,
                                      ctypes.c_size_t, _P,
                                      ctypes.POINTER(WbCosxStats)]),
        'wb_cosx_batch_workspace_bytes': (ctypes.c_size_t, [_P, _I64,
                                                            ctypes.POINTER(ctypes.c_size_t)]),
        'wb_cosx_batch_create': (_INT, [_INT, _P, _P, _P, _P, _P, _P, _P,
                                        ctypes.c_size_t, _INT, _P, _D, _INT, _P,
                                        ctypes.POINTER(_P)]),
        'wb_cosx_batch_run': (_INT, [_P, _P, _P, _P, ctypes.POINTER(WbCosxStats)]),
        'wb_cosx_batch_destroy': (_INT, [_P]),
        'wb_status_string': (ctypes.c_char_p, [_INT]),
        'wb_last_error': (ctypes.c_char_p, []),
        'wb_version': (_INT, []),
    }
    for name, (res, args) in sig.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args


def library_path():
    return _build.library_path()


def lib():
    """The loaded library (raises NativeLibraryMissing if not built)."""
    global _LIB
    if _LIB is None:
        with _LOCK:
            if _LIB is None:
                path = library_path()
                if not os.path.exists(path):
                    raise NativeLibraryMissing(
                        '%s is not built; run python -m '
                        'pyscf_wb97mv_fast_gb300.build' % path)
                handle = ctypes.CDLL(path, mode=ctypes.RTLD_GLOBAL)
                _declare(handle)
                _LIB = handle
    return _LIB


def check(status, what=''):
    if status == WB_OK:
        return
    L = lib()
    msg = (L.wb_last_error() or b'').decode(errors='replace')
    msg = '%s: %s' % (what, msg) if what else msg
    if status == WB_ERR_UNSUPPORTED:
        raise Unsupported(status, msg)
    if status == WB_ERR_OUT_OF_MEMORY:
        raise DeviceOutOfMemory(status, msg)
    raise NativeError(status, msg)


def ptr(arr):
    """Device/host address of a torch tensor or numpy array (None -> 0)."""
    if arr is None:
        return None
    if hasattr(arr, 'data_ptr'):
        return ctypes.c_void_p(arr.data_ptr())
    return arr.ctypes.data_as(ctypes.c_void_p)
