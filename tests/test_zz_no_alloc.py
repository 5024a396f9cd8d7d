"""GPU test of cuna2_compat_adjoint_noalloc_f32, the entry point for callers
that cannot allocate device memory once running (real-time loops where
cudaMalloc/cudaFree would stall the device, processes whose device memory
is owned by a framework's caching allocator, plugin hosts that forbid a
plugin from allocating).  Its scratch is a static device array inside the
library.  The tests check that:

* two calls in a row -- the first one also sets the device up -- agree with
  cuna2_compat_adjoint_f32, at the documented maximum sizes too
  (n = 131072 samples on a 131072-cell grid: every record slot, the largest
  twiddle tables) and on the largest single-CTA grid;
* the result matches the golden vector of the reference's own sources
  (f32_cfg1_n10000_ng32768) at the float parity bar;
* in a fresh process whose first library call is this entry point (so that
  the call itself sets the device up) the result matches the golden vector;
* after set-up a call leaves the device's free memory unchanged;
* sizes beyond the array's limits are refused and touch nothing.

Kept in a file of its own that pytest collects last; it passes alone in a
fresh process and after the other tests.
"""
import os
import subprocess
import sys

import numpy as np
import pytest
import torch

from conftest import GOLDEN_DIR, ROOT

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


def _noalloc(L, x, y, out, n, ng, fp):
    return L.cuna2_compat_adjoint_noalloc_f32(x.data_ptr(), y.data_ptr(), out.data_ptr(), n, ng, fp.data_ptr(),
                                              None)


def test_noalloc_matches_allocating_entry_point(native_built):
    from cunfft_adjoint_gb300 import _lib, cuna
    L = _lib.core()
    # calls in a row with different sizes: a four-step grid, a single-CTA grid
    # with fewer tiles (stale counters would show up here), the largest
    # single-CTA grid, and the documented maximum (n = 131072 fills every
    # record slot; ng = 131072 uses the largest twiddle tables)
    for n, ng, seed in ((10_000, 32768, 1), (3_000, 4096, 2), (30_000, 16384, 4), (131_072, 131_072, 5),
                        (10_000, 32768, 1)):
        x, y = _inputs(n, seed)
        fp = cuna.generate_filter_properties(x, n, ng)
        want = torch.zeros(ng, dtype=torch.complex64, device="cuda")
        _lib.check(L.cuna2_compat_adjoint_f32(x.data_ptr(), y.data_ptr(), want.data_ptr(), n, ng,
                                              fp.data_ptr(), None))
        got = torch.zeros(ng, dtype=torch.complex64, device="cuda")
        _lib.check(_noalloc(L, x, y, got, n, ng, fp))
        torch.cuda.synchronize()
        g, w = got.cpu().numpy(), want.cpu().numpy()
        assert np.all(np.isfinite(g)), (n, ng)
        assert _rel(g, w) < TOL, (n, ng)


def test_noalloc_matches_reference_golden(native_built):
    from cunfft_adjoint_gb300 import _lib, cuna
    L = _lib.core()
    case = np.load(os.path.join(GOLDEN_DIR, "f32_cfg1_n10000_ng32768.npz"))
    n, ng = len(case["x"]), int(case["ng"])
    x = torch.as_tensor(case["x"], device="cuda")
    y = torch.as_tensor(case["y"], device="cuda")
    fp = cuna.generate_filter_properties(x, n, ng)
    for _ in range(2):
        got = torch.zeros(ng, dtype=torch.complex64, device="cuda")
        _lib.check(_noalloc(L, x, y, got, n, ng, fp))
        torch.cuda.synchronize()
        assert _rel(got.cpu().numpy(), case["F"]) < TOL


def test_noalloc_allocates_nothing(native_built):
    from cunfft_adjoint_gb300 import _lib, cuna
    L = _lib.core()
    n, ng = 20_000, 65536
    x, y = _inputs(n, 6)
    fp = cuna.generate_filter_properties(x, n, ng)
    outs = [torch.zeros(ng, dtype=torch.complex64, device="cuda") for _ in range(3)]
    _lib.check(_noalloc(L, x, y, outs[0], n, ng, fp))  # set-up (if not done yet) and first use
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    for o in outs[1:]:
        _lib.check(_noalloc(L, x, y, o, n, ng, fp))
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0
    assert torch.equal(outs[1], outs[2])


_FRESH = r"""
import ctypes, sys
import numpy as np, torch
sys.path.insert(0, sys.argv[1])
from cunfft_adjoint_gb300 import _lib
case = np.load(sys.argv[2])
n, ng = len(case["x"]), int(case["ng"])
# the filter coefficients of the reference's own sources, placed on the
# device by hand, so that the first call into the library is the
# no-allocation entry point itself
E1 = torch.as_tensor(case["E1"], device="cuda")
E2 = torch.as_tensor(case["E2"], device="cuda")
E3 = torch.as_tensor(case["E3"], device="cuda")
h = _lib.FilterPropertiesF32(float(case["b"]), float(case["normfac"]), int(case["rf"]),
                             E1.data_ptr(), E2.data_ptr(), E3.data_ptr())
raw = torch.frombuffer(bytearray(bytes(h)), dtype=torch.uint8).cuda()
x = torch.as_tensor(case["x"], device="cuda")
y = torch.as_tensor(case["y"], device="cuda")
L = _lib.core()
for _ in range(2):
    out = torch.zeros(ng, dtype=torch.complex64, device="cuda")
    _lib.check(L.cuna2_compat_adjoint_noalloc_f32(x.data_ptr(), y.data_ptr(), out.data_ptr(), n, ng,
                                                  raw.data_ptr(), None))
    torch.cuda.synchronize()
    F = out.cpu().numpy()
    print("rel %.3e" % (np.linalg.norm(F - case["F"]) / np.linalg.norm(case["F"])))
"""


def test_noalloc_first_call_in_fresh_process(native_built):
    path = os.path.join(GOLDEN_DIR, "f32_cfg1_n10000_ng32768.npz")
    r = subprocess.run([sys.executable, "-c", _FRESH, ROOT, path], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr[-2000:]
    rels = [float(line.split()[1]) for line in r.stdout.splitlines() if line.startswith("rel ")]
    assert len(rels) == 2 and all(v < TOL for v in rels), r.stdout


def test_noalloc_rejects_sizes_beyond_its_limits(native_built):
    from cunfft_adjoint_gb300 import _lib, cuna
    L = _lib.core()
    x, y = _inputs(1000, 3)
    fp = cuna.generate_filter_properties(x, 1000, 2048)
    out = torch.zeros(1 << 18, dtype=torch.complex64, device="cuda")
    st = _noalloc(L, x, y, out, 1000, 1 << 18, fp)
    assert st == 3 and b"power of two" in L.cuna2_last_error()
    st = _noalloc(L, x, y, out, 1000, 3000, fp)
    assert st == 3
    big = torch.zeros(200_000, device="cuda")
    st = L.cuna2_compat_adjoint_noalloc_f32(big.data_ptr(), big.data_ptr(), out.data_ptr(), 200_000, 2048,
                                            fp.data_ptr(), None)
    assert st == 3 and b"maximum" in L.cuna2_last_error()
    torch.cuda.synchronize()
    assert torch.count_nonzero(out).item() == 0
