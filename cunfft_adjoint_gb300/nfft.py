"""Accurate-mode adjoint NFFT plans (cuna2_plan_* over ctypes).

    plan = AdjointNFFT(nf=2**20, R=4, m=12, dtype=torch.float32)
    F = plan(t, y, t0, T)     # F[k + nf/2] = sum_j y_j exp(2 pi i k x_j),
                              # x_j = (t_j - t0)/T - 1/2,  k = -nf/2 .. nf/2-1

t is a float64 CUDA tensor; y has the plan's dtype; F is complex64 (float
plans) or complex128.
"""
import ctypes

import torch

from . import _lib


class AdjointNFFT:
    @classmethod
    def for_tolerance(cls, nf, tol, t, y, t0=None, T=None, dtype=torch.float32):
        """The plan (R, m, schedule) that reaches relative error `tol` fastest
        on the representative input (t, y) (cuna2_plan_create_auto)."""
        self = cls.__new__(cls)
        self.nf, self.dtype = int(nf), dtype
        self.device = t.device
        self.cdtype = torch.complex64 if dtype == torch.float32 else torch.complex128
        self._h = ctypes.c_void_p()
        t, y, t0, T = AdjointNFFT._check(self, t, y, t0, T)
        out = torch.empty(self.nf, dtype=self.cdtype, device=t.device)
        R, m = ctypes.c_int(), ctypes.c_int()
        s = torch.cuda.current_stream(t.device).cuda_stream
        with torch.cuda.device(self.device):
            _lib.check(_lib.core().cuna2_plan_create_auto(
                ctypes.byref(self._h), _lib.F32 if dtype == torch.float32 else _lib.F64, self.nf, float(tol),
                t.data_ptr(), y.data_ptr(), out.data_ptr(), t.numel(), float(t0), float(T), s or None,
                ctypes.byref(R), ctypes.byref(m)))
        self.R, self.m = R.value, m.value
        ng, tau = ctypes.c_int64(), ctypes.c_double()
        _lib.check(_lib.core().cuna2_plan_info(self._h, ctypes.byref(ng), ctypes.byref(tau)))
        self.ng, self.tau = ng.value, tau.value
        return self

    def __init__(self, nf, R=2, m=8, dtype=torch.float32, device=None):
        if dtype not in (torch.float32, torch.float64):
            raise TypeError("dtype must be torch.float32 or torch.float64")
        self.nf, self.R, self.m, self.dtype = int(nf), int(R), int(m), dtype
        self.device = torch.device(device) if device is not None else torch.device("cuda", torch.cuda.current_device())
        self.cdtype = torch.complex64 if dtype == torch.float32 else torch.complex128
        self._h = ctypes.c_void_p()
        with torch.cuda.device(self.device):
            _lib.check(_lib.core().cuna2_plan_create(ctypes.byref(self._h),
                                                     _lib.F32 if dtype == torch.float32 else _lib.F64,
                                                     self.nf, self.R, self.m))
        ng, tau = ctypes.c_int64(), ctypes.c_double()
        _lib.check(_lib.core().cuna2_plan_info(self._h, ctypes.byref(ng), ctypes.byref(tau)))
        self.ng, self.tau = ng.value, tau.value

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            try:
                _lib.core().cuna2_plan_destroy(h)
            except Exception:
                pass
            self._h = ctypes.c_void_p()

    def __call__(self, t, y, t0=None, T=None, out=None, stream=None):
        return self.adjoint(t, y, t0, T, out, stream)

    def _check(self, t, y, t0, T):
        if t.dtype != torch.float64 or not t.is_cuda:
            raise TypeError("t must be a float64 CUDA tensor")
        if y.dtype != self.dtype or not y.is_cuda:
            raise TypeError("y must be a %s CUDA tensor" % self.dtype)
        t = t.contiguous()
        y = y.contiguous()
        if y.numel() != t.numel():
            raise ValueError("t and y differ in length")
        if t0 is None or T is None:
            lo, hi = (float(t.min()), float(t.max())) if t.numel() else (0.0, 1.0)
            t0 = lo if t0 is None else t0
            T = (hi - lo if hi > lo else 1.0) if T is None else T
        return t, y, t0, T

    def adjoint(self, t, y, t0=None, T=None, out=None, stream=None):
        t, y, t0, T = self._check(t, y, t0, T)
        n = t.numel()
        if out is None:
            out = torch.empty(self.nf, dtype=self.cdtype, device=t.device)
        s = (stream if stream is not None else torch.cuda.current_stream(t.device)).cuda_stream
        _lib.check(_lib.core().cuna2_adjoint(self._h, t.data_ptr(), y.data_ptr(), out.data_ptr(), n,
                                             float(t0), float(T), s or None))
        return out

    def bootstrap(self, t, y, nbs, seed=0, t0=None, T=None, out=None, stream=None):
        """nbs resamples with replacement of (t, y); returns (nbs, nf)."""
        t, y, t0, T = self._check(t, y, t0, T)
        if out is None:
            out = torch.empty((nbs, self.nf), dtype=self.cdtype, device=t.device)
        s = (stream if stream is not None else torch.cuda.current_stream(t.device)).cuda_stream
        _lib.check(_lib.core().cuna2_adjoint_bootstrap(self._h, t.data_ptr(), y.data_ptr(), out.data_ptr(),
                                                       t.numel(), int(nbs), seed & 0xFFFFFFFF,
                                                       float(t0), float(T), s or None))
        return out

    def multi(self, t, Y, t0=None, T=None, out=None, stream=None):
        """Several value channels Y (nchan, n) at the same times t, transformed
        together (shared binning and gridding); returns (nchan, nf)."""
        if Y.dim() != 2 or Y.shape[1] != t.numel():
            raise ValueError("Y must be (nchan, n)")
        t, _, t0, T = self._check(t, Y[0], t0, T)
        Y = Y.contiguous()
        if out is None:
            out = torch.empty((Y.shape[0], self.nf), dtype=self.cdtype, device=t.device)
        s = (stream if stream is not None else torch.cuda.current_stream(t.device)).cuda_stream
        _lib.check(_lib.core().cuna2_adjoint_multi(self._h, t.data_ptr(), Y.data_ptr(), out.data_ptr(), t.numel(),
                                                   Y.shape[0], float(t0), float(T), s or None))
        return out

    def backward(self, t, y, grad_F, t0, T, need_y=True, need_t=True, stream=None):
        """(dL/dy, dL/dt) for grad_F = dL/dRe F + i dL/dIm F (torch's convention)."""
        gy = torch.empty_like(y) if need_y else None
        gt = torch.empty_like(t) if need_t else None
        s = (stream if stream is not None else torch.cuda.current_stream(t.device)).cuda_stream
        g = grad_F.contiguous()
        if g.dtype != self.cdtype:
            g = g.to(self.cdtype)
        _lib.check(_lib.core().cuna2_adjoint_backward(
            self._h, t.data_ptr(), y.data_ptr(), g.data_ptr(), None if gy is None else gy.data_ptr(),
            None if gt is None else gt.data_ptr(), t.numel(), float(t0), float(T), s or None))
        return gy, gt

    def backward_batch(self, t, y, grad_F, t0, T, need_y=True, need_t=True, stream=None):
        """(dL/dy, dL/dt) of B series at once: t, y (B, N), grad_F (B, nf),
        t0 and T B values each (cuna2_adjoint_backward_batch)."""
        import numpy as np
        B = t.shape[0]
        t = t.contiguous()
        y = y.contiguous()
        gy = torch.empty_like(y) if need_y else None
        gt = torch.empty_like(t) if need_t else None
        g = grad_F.contiguous()
        if g.dtype != self.cdtype:
            g = g.to(self.cdtype)
        t0a = np.ascontiguousarray(np.broadcast_to(np.asarray(t0, np.float64), (B,)))
        Ta = np.ascontiguousarray(np.broadcast_to(np.asarray(T, np.float64), (B,)))
        s = (stream if stream is not None else torch.cuda.current_stream(t.device)).cuda_stream
        _lib.check(_lib.core().cuna2_adjoint_backward_batch(
            self._h, t.data_ptr(), y.data_ptr(), g.data_ptr(), None if gy is None else gy.data_ptr(),
            None if gt is None else gt.data_ptr(), t.shape[1], B, t0a.ctypes.data, Ta.ctypes.data, s or None))
        return gy, gt

    def set_graph(self, enable=True):
        """Replay each argument set's launch sequence as a CUDA graph
        (cuna2_plan_set_graph): plain, bootstrap (reused across seeds) and
        multi-channel calls."""
        _lib.check(_lib.core().cuna2_plan_set_graph(self._h, 1 if enable else 0))
        return self

    @property
    def schedule(self):
        """(log_tile, grid_method) of the tiled gridding."""
        lt, gm = ctypes.c_int(), ctypes.c_int()
        _lib.check(_lib.core().cuna2_plan_get_schedule(self._h, ctypes.byref(lt), ctypes.byref(gm)))
        return lt.value, gm.value

    def set_schedule(self, log_tile, grid_method):
        """Tiles of 2**log_tile cells, gridded in GRID_GATHER or GRID_SCATTER form."""
        _lib.check(_lib.core().cuna2_plan_set_schedule(self._h, int(log_tile), int(grid_method)))

    @property
    def binning(self):
        """BIN_GLOBAL or BIN_LOCAL (see cuna2_plan_set_binning)."""
        v = ctypes.c_int()
        _lib.check(_lib.core().cuna2_plan_get_binning(self._h, ctypes.byref(v)))
        return v.value

    @binning.setter
    def binning(self, mode):
        _lib.check(_lib.core().cuna2_plan_set_binning(self._h, int(mode)))

    def autotune(self, t, y, t0=None, T=None, reps=5, stream=None):
        """Time every admissible schedule on (t, y), keep the fastest; returns
        (log_tile, grid_method, best_ms)."""
        t, y, t0, T = self._check(t, y, t0, T)
        out = torch.empty(self.nf, dtype=self.cdtype, device=t.device)
        s = (stream if stream is not None else torch.cuda.current_stream(t.device)).cuda_stream
        ms = ctypes.c_float()
        _lib.check(_lib.core().cuna2_plan_autotune(self._h, t.data_ptr(), y.data_ptr(), out.data_ptr(), t.numel(),
                                                   float(t0), float(T), s or None, int(reps), ctypes.byref(ms)))
        return self.schedule + (ms.value,)

    def frequencies(self):
        """Integer frequency index k of each output bin."""
        return torch.arange(-self.nf // 2, self.nf // 2, dtype=torch.int64)


class BatchAdjointNFFT:
    """Adjoint NFFTs of many series of uneven length in one execution.

    Series s has ``n[s]`` samples and ``nf[s]`` outputs (``R * nf[s] / 2`` a
    power of two); samples of all series are concatenated in ``t``/``y`` and
    outputs in the returned flat tensor (``split`` gives per-series views).
    ``t0``/``T`` (per series) define ``x = (t - t0)/T - 1/2``.
    """

    @classmethod
    def for_tolerance(cls, n, nf, tol, t, y, t0=None, T=None, dtype=torch.float32, graph=False):
        """The batch plan (R, m, gridding schedule) that reaches relative error
        `tol` fastest on the representative batch (t, y)
        (cuna2_batch_plan_create_auto)."""
        import numpy as np
        self = cls.__new__(cls)
        self._setup(n, nf, dtype, t.device)
        if t.dtype != torch.float64 or y.dtype != dtype or t.numel() != int(self.n.sum()) or y.numel() != t.numel():
            raise ValueError("t (float64) and y (plan dtype) must hold the batch's concatenated samples")
        t, y = t.contiguous(), y.contiguous()
        ns = len(self.n)
        t0a = None if t0 is None else np.ascontiguousarray(t0, dtype=np.float64)
        Ta = None if T is None else np.ascontiguousarray(T, dtype=np.float64)
        out = torch.empty(int(self.nf.sum()), dtype=self.cdtype, device=t.device)
        R, m = np.zeros(ns, np.int32), np.zeros(ns, np.int32)
        s = torch.cuda.current_stream(t.device).cuda_stream
        self._h = ctypes.c_void_p()
        with torch.cuda.device(self.device):
            _lib.check(_lib.core().cuna2_batch_plan_create_auto(
                ctypes.byref(self._h), _lib.F32 if dtype == torch.float32 else _lib.F64, ns,
                self.n.ctypes.data, self.nf.ctypes.data, float(tol),
                None if t0a is None else t0a.ctypes.data, None if Ta is None else Ta.ctypes.data,
                t.data_ptr(), y.data_ptr(), out.data_ptr(), s or None, R.ctypes.data, m.ctypes.data))
        self.R, self.m = R, m  # per series
        if graph:
            _lib.check(_lib.core().cuna2_batch_set_graph(self._h, 1))
        return self

    def _setup(self, n, nf, dtype, device):
        import numpy as np
        self.n = np.ascontiguousarray(n, dtype=np.int64)
        self.nf = np.ascontiguousarray(nf, dtype=np.int64)
        if self.n.shape != self.nf.shape or self.n.ndim != 1:
            raise ValueError("n and nf must be 1-D and of equal length")
        self.dtype = dtype
        self.cdtype = torch.complex64 if dtype == torch.float32 else torch.complex128
        self.device = torch.device(device) if device is not None else torch.device("cuda", torch.cuda.current_device())
        self.f_off = np.concatenate([[0], np.cumsum(self.nf)])
        self.s_off = np.concatenate([[0], np.cumsum(self.n)])

    def __init__(self, n, nf, R=2, m=8, t0=None, T=None, dtype=torch.float32, device=None, graph=False):
        """R and m: one value for every series, or one per series."""
        import numpy as np
        self._setup(n, nf, dtype, device)
        ns = len(self.n)
        self.R = np.ascontiguousarray(np.broadcast_to(np.asarray(R), (ns,)), dtype=np.int32)
        self.m = np.ascontiguousarray(np.broadcast_to(np.asarray(m), (ns,)), dtype=np.int32)
        t0a = None if t0 is None else np.ascontiguousarray(t0, dtype=np.float64)
        Ta = None if T is None else np.ascontiguousarray(T, dtype=np.float64)
        self._h = ctypes.c_void_p()
        with torch.cuda.device(self.device):
            _lib.check(_lib.core().cuna2_batch_plan_create_ex(
                ctypes.byref(self._h), _lib.F32 if dtype == torch.float32 else _lib.F64, ns,
                self.n.ctypes.data, self.nf.ctypes.data, self.R.ctypes.data, self.m.ctypes.data,
                None if t0a is None else t0a.ctypes.data, None if Ta is None else Ta.ctypes.data))
        if graph:
            _lib.check(_lib.core().cuna2_batch_set_graph(self._h, 1))

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            try:
                _lib.core().cuna2_batch_plan_destroy(h)
            except Exception:
                pass
            self._h = ctypes.c_void_p()

    def set_times(self, t0, T):
        import numpy as np
        t0a = np.ascontiguousarray(t0, dtype=np.float64)
        Ta = np.ascontiguousarray(T, dtype=np.float64)
        _lib.check(_lib.core().cuna2_batch_set_times(self._h, t0a.ctypes.data, Ta.ctypes.data))

    def __call__(self, t, y, out=None, stream=None):
        if t.dtype != torch.float64 or y.dtype != self.dtype or not (t.is_cuda and y.is_cuda):
            raise TypeError("t must be float64 and y %s CUDA tensors" % self.dtype)
        if t.numel() != int(self.s_off[-1]) or y.numel() != t.numel():
            raise ValueError("t and y must hold sum(n) samples")
        t = t.contiguous()
        y = y.contiguous()
        if out is None:
            out = torch.empty(int(self.f_off[-1]), dtype=self.cdtype, device=t.device)
        s = (stream if stream is not None else torch.cuda.current_stream(t.device)).cuda_stream
        _lib.check(_lib.core().cuna2_batch_adjoint(self._h, t.data_ptr(), y.data_ptr(), out.data_ptr(), s or None))
        return out

    def split(self, F):
        return [F[int(self.f_off[i]):int(self.f_off[i + 1])] for i in range(len(self.nf))]

    @property
    def schedule(self):
        """(log_tile, grid_method) of the large series' gridding."""
        lt, gm = ctypes.c_int(), ctypes.c_int()
        _lib.check(_lib.core().cuna2_batch_get_schedule(self._h, ctypes.byref(lt), ctypes.byref(gm)))
        return lt.value, gm.value

    def set_schedule(self, log_tile, grid_method):
        _lib.check(_lib.core().cuna2_batch_set_schedule(self._h, int(log_tile), int(grid_method)))

    def autotune(self, t, y, reps=3, stream=None):
        """Time every admissible schedule on (t, y), keep the fastest;
        returns (log_tile, grid_method, best_ms)."""
        out = torch.empty(int(self.f_off[-1]), dtype=self.cdtype, device=t.device)
        s = (stream if stream is not None else torch.cuda.current_stream(t.device)).cuda_stream
        ms = ctypes.c_float()
        _lib.check(_lib.core().cuna2_batch_autotune(self._h, t.contiguous().data_ptr(), y.contiguous().data_ptr(),
                                                    out.data_ptr(), s or None, int(reps), ctypes.byref(ms)))
        return self.schedule + (ms.value,)
