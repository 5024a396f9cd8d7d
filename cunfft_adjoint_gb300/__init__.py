"""GB300-native adjoint NFFT (drop-in for CUNA / johnh2o2/cunfft_adjoint).

Native code lives in cunfft_adjoint_gb300/lib (built by
``python -m cunfft_adjoint_gb300.build``):

* libcuna_gb300.so -- sm_103a kernels and the extern "C" cuna2_* API
* libcunaf.so / libcunad.so -- the reference's C++ API, same symbol names

Python front ends: ``cuna`` (the reference's function names over torch
tensors) and ``nfft.AdjointNFFT`` (accurate-mode plans).
"""
from . import _lib  # noqa: F401
from ._lib import CunaError  # noqa: F401

__all__ = ["CunaError", "cuna", "nfft"]
