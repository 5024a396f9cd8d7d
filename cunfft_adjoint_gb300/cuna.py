"""Python mirror of the reference library's interface (CUNA v1.3, inc/cuna.h
and inc/cuna_filter.h) over the GB300 C-ABI.

Same function names and argument meaning as the reference; arrays are torch
CUDA tensors (device pointers in the reference) or numpy arrays for the
host-array convenience call.  Where the reference terminates the process on a
failed call, these raise ``CunaError``.

    fp = generate_filter_properties(x, n, ng)              # src/gaussian_filter.cu:102
    cunfft_adjoint_raw(x, y, f_hat, n, ng, fp)              # src/cuna_kernel.cu:148
    cunfft_adjoint_raw_async(x, y, f_hat, n, ng, fp, s)     # src/cuna_kernel.cu:186
    cunfft_adjoint_raw_async_bootstrap(x, y, f_hat, n, ng, nbs, fp, s, seed)
                                                            # src/cuna_kernel.cu:236
    F = cunfft_adjoint(x, y, ng)                            # src/cuna.cpp:38
"""
import ctypes

import numpy as np
import torch

from . import _lib

FILTER_RADIUS = {torch.float32: 6, torch.float64: 12}  # src/gaussian_filter.cu:29-33


def _stream_handle(stream):
    if stream is None:
        return None
    if isinstance(stream, int):
        return stream or None
    return stream.cuda_stream or None


def _ptr(t):
    return None if t is None else t.data_ptr()


def _suffix(dtype):
    if dtype == torch.float32:
        return "f32"
    if dtype == torch.float64:
        return "f64"
    raise TypeError("CUNA supports float32 and float64, got %s" % dtype)


def _ctype(dtype):
    return torch.complex64 if dtype == torch.float32 else torch.complex128


class FilterProperties:
    """Host and device copies of the reference's filter_properties.

    ``host`` is the ctypes struct (b, normfac, filter_radius, E1/E2/E3 device
    pointers); ``device`` is a CUDA tensor holding the same bytes, whose
    data_ptr() is the ``const filter_properties *`` the transforms take.
    """

    def __init__(self, n, dtype, device):
        self.dtype = dtype
        self.n = n
        rf = FILTER_RADIUS[dtype]
        self.E1 = torch.empty(max(n, 1), dtype=dtype, device=device)
        self.E2 = torch.empty(max(n, 1), dtype=dtype, device=device)
        self.E3 = torch.empty(rf, dtype=dtype, device=device)
        S = _lib.FilterPropertiesF32 if dtype == torch.float32 else _lib.FilterPropertiesF64
        self.host = S()
        self.host.E1, self.host.E2, self.host.E3 = _ptr(self.E1), _ptr(self.E2), _ptr(self.E3)
        self.device = torch.zeros(ctypes.sizeof(S), dtype=torch.uint8, device=device)

    @property
    def b(self):
        return self.host.b

    @property
    def normfac(self):
        return self.host.normfac

    @property
    def filter_radius(self):
        return self.host.filter_radius

    def data_ptr(self):
        return self.device.data_ptr()


def generate_pinned_filter_properties(x, n, ng, fprops, stream=None):
    """Fill a caller-allocated FilterProperties on `stream` (asynchronous)."""
    fn = getattr(_lib.core(), "cuna2_compat_filter_" + _suffix(x.dtype))
    _lib.check(fn(_ptr(x), n, ng, ctypes.byref(fprops.host), fprops.data_ptr(), _stream_handle(stream)))
    return fprops


def generate_filter_properties(x, n, ng):
    """Allocate and compute the filter for device positions x (synchronous)."""
    fp = FilterProperties(n, x.dtype, x.device)
    generate_pinned_filter_properties(x, n, ng, fp, None)
    torch.cuda.synchronize(x.device)
    return fp


def free_filter_properties(fprops):
    """Release the device memory of `fprops` (kept for API symmetry)."""
    fprops.E1 = fprops.E2 = fprops.E3 = fprops.device = None


def cunfft_adjoint_raw_async(x, f_data, f_hat, n, ng, gpu_fprops, stream=None):
    """Gridding -> inverse FFT -> deconvolution into f_hat (ng complex values,
    accumulating: zero it first).  f_data=None grids y = 1."""
    fn = getattr(_lib.core(), "cuna2_compat_adjoint_" + _suffix(x.dtype))
    _lib.check(fn(_ptr(x), _ptr(f_data), _ptr(f_hat), n, ng, gpu_fprops.data_ptr(), _stream_handle(stream)))


def cunfft_adjoint_raw(x, f_data, f_hat, n, ng, gpu_fprops):
    """cunfft_adjoint_raw_async on the default stream."""
    cunfft_adjoint_raw_async(x, f_data, f_hat, n, ng, gpu_fprops, None)


def cunfft_adjoint_raw_async_bootstrap(x, f_data, f_hat, n, ng, nbs, gpu_fprops, stream=None, seed=0):
    """nbs bootstrap resamples into f_hat (nbs x ng complex, accumulating)."""
    fn = getattr(_lib.core(), "cuna2_compat_bootstrap_" + _suffix(x.dtype))
    _lib.check(fn(_ptr(x), _ptr(f_data), _ptr(f_hat), n, ng, nbs, gpu_fprops.data_ptr(),
                  seed & 0xFFFFFFFF, _stream_handle(stream)))


def cunfft_adjoint(x, f, ng, flags=0):
    """Host arrays in, host complex array of ng values out (src/cuna.cpp:38)."""
    x = np.asarray(x)
    dtype = torch.float32 if x.dtype == np.float32 else torch.float64
    xd = torch.as_tensor(np.ascontiguousarray(x, dtype=x.dtype), device="cuda")
    fd = None if f is None else torch.as_tensor(np.ascontiguousarray(f, dtype=x.dtype), device="cuda")
    n = len(x)
    fp = generate_filter_properties(xd, n, ng)
    out = torch.zeros(ng, dtype=_ctype(dtype), device="cuda")
    cunfft_adjoint_raw(xd, fd, out, n, ng, fp)
    return out.cpu().numpy()
