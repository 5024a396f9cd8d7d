"""Generalised Lomb-Scargle periodogram on the GPU (cuna2_lomb_scargle).

    P = lomb_scargle(t, y, dy=None, nfreq=..., df=...)   # P[k] at f = (k + 1) df

Floating-mean periodogram (Zechmeister & Kuerster 2009) with weights 1/dy^2;
the trigonometric sums come from one two-channel adjoint NFFT.
"""
import torch

from . import _lib


def lomb_scargle(t, y, dy=None, nfreq=None, df=None, t0=None, R=2, m=8, out=None, stream=None):
    if t.dtype != torch.float64 or not t.is_cuda:
        raise TypeError("t must be a float64 CUDA tensor")
    if y.dtype not in (torch.float32, torch.float64) or not y.is_cuda:
        raise TypeError("y must be a float32 or float64 CUDA tensor")
    t = t.contiguous()
    y = y.contiguous()
    if dy is not None:
        dy = dy.to(y.dtype).contiguous()
    if t0 is None:
        t0 = float(t.min())
    if df is None:
        df = 1.0 / (5.0 * float(t.max() - t.min()))  # oversampling 5
    if nfreq is None:
        raise ValueError("nfreq is required")
    if out is None:
        out = torch.empty(int(nfreq), dtype=y.dtype, device=t.device)
    s = (stream if stream is not None else torch.cuda.current_stream(t.device)).cuda_stream
    dt = _lib.F32 if y.dtype == torch.float32 else _lib.F64
    _lib.check(_lib.core().cuna2_lomb_scargle(dt, t.data_ptr(), y.data_ptr(), None if dy is None else dy.data_ptr(),
                                              t.numel(), int(nfreq), float(df), float(t0), int(R), int(m),
                                              out.data_ptr(), s or None))
    return out
