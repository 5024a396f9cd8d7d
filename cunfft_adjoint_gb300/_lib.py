"""ctypes bindings of the native libraries (cunfft_adjoint_gb300/lib/*.so).

The product path is the native library: if it is missing this module raises
instead of falling back to anything else.  Build it with
``python -m cunfft_adjoint_gb300.build`` (or ``__graft_entry__.build()``).
"""
import ctypes
import os

LIB_DIR = os.path.join(os.path.dirname(os.path.abspath(__file__)), "lib")

_P = ctypes.c_void_p
_I = ctypes.c_int
_I64 = ctypes.c_int64
_D = ctypes.c_double
_U = ctypes.c_uint

SUCCESS = 0
STATUS = {0: "CUNA2_SUCCESS", 1: "CUNA2_ERROR_INVALID_VALUE", 2: "CUNA2_ERROR_CUDA",
          3: "CUNA2_ERROR_UNSUPPORTED", 4: "CUNA2_ERROR_ALLOC", 5: "CUNA2_ERROR_CUFFT"}
F32, F64 = 0, 1
GRID_GATHER, GRID_SCATTER, GRID_FIXED = 0, 1, 2
BIN_GLOBAL, BIN_LOCAL = 0, 1


class CunaError(RuntimeError):
    """A cuna2_* call returned a non-zero status."""

    def __init__(self, status, message):
        super().__init__("%s: %s" % (STATUS.get(status, status), message))
        self.status = status


class FilterPropertiesF32(ctypes.Structure):
    """Layout of the reference's float filter_properties (40 bytes)."""
    _fields_ = [("b", ctypes.c_float), ("normfac", ctypes.c_float), ("filter_radius", _I),
                ("E1", _P), ("E2", _P), ("E3", _P)]


class FilterPropertiesF64(ctypes.Structure):
    """Layout of the reference's double filter_properties (48 bytes)."""
    _fields_ = [("b", ctypes.c_double), ("normfac", ctypes.c_double), ("filter_radius", _I),
                ("E1", _P), ("E2", _P), ("E3", _P)]


# name -> (restype, argtypes)
CORE_SIGNATURES = {
    "cuna2_last_error": (ctypes.c_char_p, []),
    "cuna2_status_string": (ctypes.c_char_p, [_I]),
    "cuna2_version": (ctypes.c_char_p, []),
    "cuna2_wait_timeouts": (ctypes.c_longlong, []),
    "cuna2_compat_filter_radius": (_I, [_I]),
    "cuna2_compat_filter_f32": (_I, [_P, _I, _I, _P, _P, _P]),
    "cuna2_compat_filter_f64": (_I, [_P, _I, _I, _P, _P, _P]),
    "cuna2_compat_adjoint_f32": (_I, [_P, _P, _P, _I, _I, _P, _P]),
    "cuna2_compat_adjoint_f64": (_I, [_P, _P, _P, _I, _I, _P, _P]),
    "cuna2_compat_bootstrap_f32": (_I, [_P, _P, _P, _I, _I, _I, _P, _U, _P]),
    "cuna2_compat_bootstrap_f64": (_I, [_P, _P, _P, _I, _I, _I, _P, _U, _P]),
    "cuna2_compat_grid_f32": (_I, [_P, _P, _P, _I, _I, _P, _P]),
    "cuna2_compat_grid_f64": (_I, [_P, _P, _P, _I, _I, _P, _P]),
    "cuna2_compat_fft_f32": (_I, [_P, _I, _I, _P, _I, _P]),
    "cuna2_compat_fft_f64": (_I, [_P, _I, _I, _P, _I, _P]),
    "cuna2_compat_normalize_f32": (_I, [_P, _I, _I, _P, _P]),
    "cuna2_compat_normalize_f64": (_I, [_P, _I, _I, _P, _P]),
    "cuna2_compat_adjoint_noalloc_f32": (_I, [_P, _P, _P, _I, _I, _P, _P]),
    "cuna2_plan_create": (_I, [_P, _I, _I64, _I, _I]),
    "cuna2_plan_destroy": (_I, [_P]),
    "cuna2_plan_info": (_I, [_P, _P, _P]),
    "cuna2_adjoint": (_I, [_P, _P, _P, _P, _I64, _D, _D, _P]),
    "cuna2_adjoint_host": (_I, [_P, _P, _P, _P, _I64, _D, _D, _P]),
    "cuna2_adjoint_host_async": (_I, [_P, _P, _P, _P, _I64, _D, _D, _P]),
    "cuna2_adjoint_bootstrap": (_I, [_P, _P, _P, _P, _I64, _I, _U, _D, _D, _P]),
    "cuna2_adjoint_backward": (_I, [_P, _P, _P, _P, _P, _P, _I64, _D, _D, _P]),
    "cuna2_adjoint_backward_batch": (_I, [_P, _P, _P, _P, _P, _P, _I64, _I, _P, _P, _P]),
    "cuna2_adjoint_multi": (_I, [_P, _P, _P, _P, _I64, _I, _D, _D, _P]),
    "cuna2_lomb_scargle": (_I, [_I, _P, _P, _P, _I64, _I64, _D, _D, _I, _I, _P, _P]),
    "cuna2_plan_set_graph": (_I, [_P, _I]),
    "cuna2_plan_set_schedule": (_I, [_P, _I, _I]),
    "cuna2_plan_set_binning": (_I, [_P, _I]),
    "cuna2_plan_create_auto": (_I, [_P, _I, _I64, _D, _P, _P, _P, _I64, _D, _D, _P, _P, _P]),
    "cuna2_plan_get_binning": (_I, [_P, _P]),
    "cuna2_plan_get_schedule": (_I, [_P, _P, _P]),
    "cuna2_plan_autotune": (_I, [_P, _P, _P, _P, _I64, _D, _D, _P, _I, _P]),
    "cuna2_plan_profile": (_I, [_P, _P, _P, _P, _I64, _D, _D, _P, _P, _P, _I, _P]),
    "cuna2_plan_time_grid": (_I, [_P, _P, _P, _P, _I64, _D, _D, _I, _P, _P]),
    "cuna2_batch_plan_create": (_I, [_P, _I, _I, _P, _P, _I, _I, _P, _P]),
    "cuna2_batch_plan_create_auto": (_I, [_P, _I, _I, _P, _P, _D, _P, _P, _P, _P, _P, _P, _P, _P]),
    "cuna2_batch_plan_create_ex": (_I, [_P, _I, _I, _P, _P, _P, _P, _P, _P]),
    "cuna2_batch_get_filter": (_I, [_P, _P, _P]),
    "cuna2_batch_plan_destroy": (_I, [_P]),
    "cuna2_batch_set_times": (_I, [_P, _P, _P]),
    "cuna2_batch_info": (_I, [_P, _P, _P]),
    "cuna2_batch_set_graph": (_I, [_P, _I]),
    "cuna2_batch_adjoint": (_I, [_P, _P, _P, _P, _P]),
    "cuna2_batch_set_schedule": (_I, [_P, _I, _I]),
    "cuna2_batch_get_schedule": (_I, [_P, _P, _P]),
    "cuna2_batch_autotune": (_I, [_P, _P, _P, _P, _P, _I, _P]),
    "cuna2_inspect_compat_taps_f32": (_I, [_P, _I, _I, _I, _P, _P, _P, _P, _P]),
    "cuna2_inspect_compat_taps_f64": (_I, [_P, _I, _I, _I, _P, _P, _P, _P, _P]),
    "cuna2_inspect_bootstrap_draws": (_I, [_I, _I, _U, _P, _P]),
    "cuna2_inspect_compat_bins_f32": (_I, [_P, _P, _I, _I, _P, _I, _P, _P, _I, _P, _P]),
    "cuna2_inspect_compat_bins_f64": (_I, [_P, _P, _I, _I, _P, _I, _P, _P, _I, _P, _P]),
    "cuna2_inspect_phases": (_I, [_P, _I64, _D, _D, _I64, _P, _P, _P]),
    "cuna2_plan_inspect_bins": (_I, [_P, _P, _P, _I64, _D, _D, _P, _P, _I64, _P, _P]),
}

_core = None
_dropin = {}


def _load(name):
    path = os.path.join(LIB_DIR, name)
    if not os.path.exists(path):
        raise ImportError("native library %s is missing; build it with "
                          "`python -m cunfft_adjoint_gb300.build`" % path)
    return ctypes.CDLL(path)


def core():
    """The core library with every cuna2_* signature declared."""
    global _core
    if _core is None:
        lib = _load("libcuna_gb300.so")
        for name, (res, args) in CORE_SIGNATURES.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _core = lib
    return _core


def dropin(prec):
    """libcunaf.so ('f') or libcunad.so ('d'), the CUNA-compatible libraries."""
    if prec not in _dropin:
        _dropin[prec] = _load("libcuna%s.so" % prec)
    return _dropin[prec]


def check(status):
    if status != SUCCESS:
        msg = core().cuna2_last_error()
        raise CunaError(status, msg.decode() if msg else "")
    return status


def library_paths():
    return [os.path.join(LIB_DIR, n) for n in ("libcuna_gb300.so", "libcunaf.so", "libcunad.so")]
