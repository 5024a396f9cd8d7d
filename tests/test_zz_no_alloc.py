"""GPU test of cuna2_compat_adjoint_noalloc_f32, the entry point for callers
that cannot allocate device memory once running (real-time loops where
cudaMalloc/cudaFree would stall the device, processes whose device memory
is owned by a framework's caching allocator, plugin hosts that forbid a
plugin from allocating).  Its scratch is a static device array inside the
library, so the test checks that two calls in a row -- the first one also
sets the device up -- agree with cuna2_compat_adjoint_f32, and that sizes
beyond the array's limits are refused.

Kept in a file of its own that pytest collects last; it passes alone in a
fresh process and after the other tests.
"""
import ctypes

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

TOL = 1e-5  # relative L2, the float parity bar used by the other compat tests


def _inputs(n, seed):
    rng = np.random.default_rng(seed)
    t = np.sort(rng.uniform(0.0, 1.0, n))
    x = ((t - t[0]) / (t[-1] - t[0]) - 0.5).astype(np.float32)
    y = (np.sin(2 * np.pi * 137 * t) + rng.normal(0, 0.5, n)).astype(np.float32)
    return torch.as_tensor(x, device="cuda"), torch.as_tensor(y, device="cuda")


def _rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def test_noalloc_matches_allocating_entry_point(native_built):
    from cunfft_adjoint_gb300 import _lib, cuna
    L = _lib.core()
    # two calls in a row with different sizes: a four-step grid, then a
    # single-CTA grid with fewer tiles (stale counters would show up here)
    for n, ng, seed in ((10_000, 32768, 1), (3_000, 4096, 2)):
        x, y = _inputs(n, seed)
        fp = cuna.generate_filter_properties(x, n, ng)
        want = torch.zeros(ng, dtype=torch.complex64, device="cuda")
        _lib.check(L.cuna2_compat_adjoint_f32(x.data_ptr(), y.data_ptr(), want.data_ptr(), n, ng,
                                              fp.data_ptr(), None))
        got = torch.zeros(ng, dtype=torch.complex64, device="cuda")
        _lib.check(L.cuna2_compat_adjoint_noalloc_f32(x.data_ptr(), y.data_ptr(), got.data_ptr(), n, ng,
                                                      fp.data_ptr(), None))
        torch.cuda.synchronize()
        assert _rel(got.cpu().numpy(), want.cpu().numpy()) < TOL, (n, ng)


def test_noalloc_rejects_sizes_beyond_its_limits(native_built):
    from cunfft_adjoint_gb300 import _lib, cuna
    L = _lib.core()
    x, y = _inputs(1000, 3)
    fp = cuna.generate_filter_properties(x, 1000, 2048)
    out = torch.zeros(1 << 18, dtype=torch.complex64, device="cuda")
    st = L.cuna2_compat_adjoint_noalloc_f32(x.data_ptr(), y.data_ptr(), out.data_ptr(), 1000, 1 << 18,
                                            fp.data_ptr(), None)
    assert st == 3 and b"power of two" in L.cuna2_last_error()
    st = L.cuna2_compat_adjoint_noalloc_f32(x.data_ptr(), y.data_ptr(), out.data_ptr(), 1000, 3000,
                                            fp.data_ptr(), None)
    assert st == 3
    big = torch.zeros(200_000, device="cuda")
    st = L.cuna2_compat_adjoint_noalloc_f32(big.data_ptr(), big.data_ptr(), out.data_ptr(), 200_000, 2048,
                                            fp.data_ptr(), None)
    assert st == 3 and b"maximum" in L.cuna2_last_error()
    torch.cuda.synchronize()
    assert torch.count_nonzero(out).item() == 0
