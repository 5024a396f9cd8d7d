"""GPU parity of compat mode (the reference's arithmetic) through the C-ABI,
against the golden vectors of the reference's own sources and the oracle.

Tolerances (relative L2 over all bins): 1e-5 float, 1e-12 double, the
parity bar for the reference's libcunaf / libcunad builds.  Non power-of-two
grids: the reference's GPU build contracts ng*x - u into one FMA
(src/gaussian_filter.cu:213-217), which the CPU-built golden vectors do not,
so those compare at 1e-5 against the oracle (which contracts) and 5e-5
against the golden file.
"""
import ctypes

import numpy as np
import pytest
import torch

from conftest import golden_cases, rel_l2

pytestmark = pytest.mark.gpu

PLAIN = golden_cases("plain")
BOOT = golden_cases("boot")


def _tol(dt):
    return 1e-5 if dt == np.float32 else 1e-12


def _pow2(ng):
    return ng & (ng - 1) == 0


@pytest.fixture(scope="module")
def cuna(native_built):
    from cunfft_adjoint_gb300 import cuna as C
    return C


def _dev(a):
    return None if a is None else torch.as_tensor(np.ascontiguousarray(a), device="cuda")


def _ctype(dt):
    return torch.complex64 if dt == np.float32 else torch.complex128


@pytest.mark.parametrize("case", PLAIN, ids=lambda c: c["name"])
def test_filter_properties(cuna, case):
    x = _dev(case["x"])
    n, ng = len(case["x"]), int(case["ng"])
    fp = cuna.generate_filter_properties(x, n, ng)
    assert fp.b == case["b"] and fp.normfac == case["normfac"] and fp.filter_radius == case["rf"]
    tol = 3e-5 if case["x"].dtype == np.float32 else 1e-14
    if not _pow2(ng):
        tol = 2e-3  # FMA contraction shifts eps by one ulp of ng*x (see module doc)
    for k in ("E1", "E2"):
        got = getattr(fp, k)[:n].cpu().numpy()
        assert np.max(np.abs(got / case[k] - 1)) < tol, k
    assert np.max(np.abs(fp.E3.cpu().numpy() / case["E3"] - 1)) < max(tol, 3e-5)


@pytest.mark.parametrize("case", PLAIN, ids=lambda c: c["name"])
def test_adjoint_raw_parity(cuna, oracle_lib, case):
    dt = case["x"].dtype
    x, y = _dev(case["x"]), _dev(case.get("y"))
    n, ng = len(case["x"]), int(case["ng"])
    fp = cuna.generate_filter_properties(x, n, ng)
    f0 = case.get("f_hat0")
    f_hat = _dev(f0) if f0 is not None else torch.zeros(ng, dtype=_ctype(dt), device="cuda")
    cuna.cunfft_adjoint_raw(x, y, f_hat, n, ng, fp)
    got = f_hat.cpu().numpy()
    ora = oracle_lib.compat_adjoint(case["x"], case.get("y"), ng, "f" if dt == np.float32 else "d", f0)
    assert rel_l2(got, ora) < _tol(dt)
    assert rel_l2(got, case["F"]) < (_tol(dt) if _pow2(ng) else 5e-5)


@pytest.mark.parametrize("case", PLAIN[:4], ids=lambda c: c["name"])
def test_adjoint_async_stream(cuna, case):
    dt = case["x"].dtype
    x, y = _dev(case["x"]), _dev(case.get("y"))
    n, ng = len(case["x"]), int(case["ng"])
    s = torch.cuda.Stream()
    fp = cuna.FilterProperties(n, x.dtype, x.device)
    f0 = case.get("f_hat0")
    with torch.cuda.stream(s):
        cuna.generate_pinned_filter_properties(x, n, ng, fp, s)
        f_hat = _dev(f0) if f0 is not None else torch.zeros(ng, dtype=_ctype(dt), device="cuda")
        cuna.cunfft_adjoint_raw_async(x, y, f_hat, n, ng, fp, s)
    s.synchronize()
    assert rel_l2(f_hat.cpu().numpy(), case["F"]) < (_tol(dt) if _pow2(ng) else 5e-5)


@pytest.mark.parametrize("case", BOOT, ids=lambda c: c["name"])
def test_bootstrap_parity(cuna, oracle_lib, case):
    dt = case["x"].dtype
    x, y = _dev(case["x"]), _dev(case.get("y"))
    n, ng, nbs, seed = len(case["x"]), int(case["ng"]), int(case["nbs"]), int(case["seed"])
    fp = cuna.generate_filter_properties(x, n, ng)
    f_hat = torch.zeros(nbs * ng, dtype=_ctype(dt), device="cuda")
    cuna.cunfft_adjoint_raw_async_bootstrap(x, y, f_hat, n, ng, nbs, fp, None, seed)
    torch.cuda.synchronize()
    got = f_hat.cpu().numpy().reshape(nbs, ng)
    assert rel_l2(got, case["F"]) < _tol(dt)


def test_stages_compose(cuna, native_built):
    """performGridding + performFFTs + normalizeResults == the fused call."""
    from cunfft_adjoint_gb300 import _lib
    case = [c for c in PLAIN if c["name"].startswith("f32_n1000")][0]
    x, y = _dev(case["x"]), _dev(case["y"])
    n, ng = len(case["x"]), int(case["ng"])
    fp = cuna.generate_filter_properties(x, n, ng)
    L = _lib.core()
    g = torch.zeros(ng, dtype=torch.complex64, device="cuda")
    _lib.check(L.cuna2_compat_grid_f32(x.data_ptr(), y.data_ptr(), g.data_ptr(), n, ng, fp.data_ptr(), None))
    torch.cuda.synchronize()
    assert rel_l2(g.cpu().numpy(), case["grid"]) < 1e-5
    _lib.check(L.cuna2_compat_fft_f32(g.data_ptr(), ng, 1, fp.data_ptr(), 0, None))
    _lib.check(L.cuna2_compat_normalize_f32(g.data_ptr(), ng, 1, fp.data_ptr(), None))
    torch.cuda.synchronize()
    assert rel_l2(g.cpu().numpy(), case["F"]) < 1e-5


@pytest.mark.parametrize("prec,n,ng", [("f", 1_000_000, 1 << 22), ("d", 200_000, 1 << 19),
                                       ("f", 50_000, 1 << 16), ("f", 3000, 5000)])
def test_large_grids_vs_oracle(cuna, oracle_lib, prec, n, ng):
    """Four-step FFT sizes (and a non power-of-two grid on the cuFFT path)
    at reference-scale inputs, against the oracle."""
    dt = np.float32 if prec == "f" else np.float64
    rng = np.random.default_rng(n + ng)
    t = rng.uniform(0, 1, n)
    x = ((t - t.min()) / (t.max() - t.min()) - 0.5).astype(dt)
    y = (np.sin(2 * np.pi * 41.3 * t) + rng.normal(0, 1, n)).astype(dt)
    xd, yd = _dev(x), _dev(y)
    fp = cuna.generate_filter_properties(xd, n, ng)
    f_hat = torch.zeros(ng, dtype=_ctype(dt), device="cuda")
    cuna.cunfft_adjoint_raw(xd, yd, f_hat, n, ng, fp)
    got = f_hat.cpu().numpy()
    ora = oracle_lib.compat_adjoint(x, y, ng, prec)
    assert rel_l2(got, ora) < _tol(dt)


def test_bootstrap_cfg3_shape(cuna, oracle_lib):
    """Bootstrap at the reference-scale grid (ng = 65536), 16 resamples."""
    n, ng, nbs, seed = 5000, 65536, 16, 2024
    rng = np.random.default_rng(3)
    t = rng.uniform(0, 100, n)
    x = ((t - t.min()) / (t.max() - t.min()) - 0.5).astype(np.float32)
    y = (np.sin(2 * np.pi * t / 2.1) + rng.normal(0, 0.3, n)).astype(np.float32)
    xd, yd = _dev(x), _dev(y)
    fp = cuna.generate_filter_properties(xd, n, ng)
    f_hat = torch.zeros(nbs * ng, dtype=torch.complex64, device="cuda")
    cuna.cunfft_adjoint_raw_async_bootstrap(xd, yd, f_hat, n, ng, nbs, fp, None, seed)
    torch.cuda.synchronize()
    ora = oracle_lib.compat_bootstrap(x, y, ng, nbs, seed, "f")
    assert rel_l2(f_hat.cpu().numpy().reshape(nbs, ng), ora) < 1e-5


def test_rerun_is_stable(cuna):
    case = [c for c in PLAIN if c["name"].startswith("f32_cfg1")][0]
    x, y = _dev(case["x"]), _dev(case["y"])
    n, ng = len(case["x"]), int(case["ng"])
    fp = cuna.generate_filter_properties(x, n, ng)
    outs = []
    for _ in range(3):
        f_hat = torch.zeros(ng, dtype=torch.complex64, device="cuda")
        cuna.cunfft_adjoint_raw(x, y, f_hat, n, ng, fp)
        outs.append(f_hat.cpu().numpy())
    assert rel_l2(outs[1], outs[0]) < 1e-6 and rel_l2(outs[2], outs[0]) < 1e-6


def test_dropin_results_are_bit_reproducible(cuna):
    """The drop-in sums each grid tile in fixed point with integer atomics,
    so, unlike the reference's float atomics, repeated calls give identical
    bits: a plain transform of 200,000 samples on 2^20 cells (three calls)
    and a 64-resample bootstrap (two calls)."""
    rng = np.random.default_rng(17)
    n, ng = 200_000, 1 << 20
    x = _dev(rng.uniform(-0.5, 0.5, n).astype(np.float32))
    y = _dev(rng.normal(0, 1, n).astype(np.float32))
    fp = cuna.generate_filter_properties(x, n, ng)
    outs = []
    for _ in range(3):
        f_hat = torch.zeros(ng, dtype=torch.complex64, device="cuda")
        cuna.cunfft_adjoint_raw(x, y, f_hat, n, ng, fp)
        outs.append(f_hat.cpu().numpy())
    assert np.array_equal(outs[0], outs[1]) and np.array_equal(outs[0], outs[2])
    n2, ng2, nbs = 5000, 1 << 16, 64
    x2 = _dev(rng.uniform(-0.5, 0.5, n2).astype(np.float32))
    y2 = _dev(rng.normal(0, 1, n2).astype(np.float32))
    fp2 = cuna.generate_filter_properties(x2, n2, ng2)
    boots = []
    for _ in range(2):
        fb = torch.zeros(nbs * ng2, dtype=torch.complex64, device="cuda")
        cuna.cunfft_adjoint_raw_async_bootstrap(x2, y2, fb, n2, ng2, nbs, fp2, seed=3)
        torch.cuda.synchronize()
        boots.append(fb.cpu().numpy())
    assert np.array_equal(boots[0], boots[1])


def test_invalid_arguments_raise(cuna):
    from cunfft_adjoint_gb300 import CunaError
    x = torch.zeros(10, device="cuda")
    fp = cuna.generate_filter_properties(torch.linspace(-0.5, 0.5, 10, device="cuda"), 10, 64)
    f_hat = torch.zeros(64, dtype=torch.complex64, device="cuda")
    with pytest.raises(CunaError) as e:
        cuna.cunfft_adjoint_raw(x, None, f_hat, -1, 64, fp)
    assert e.value.status == 1
    with pytest.raises(CunaError):
        cuna.cunfft_adjoint_raw(x, None, f_hat, 10, 0, fp)


# ---------------------------------------------------------------------------
# the drop-in libraries, called by their C++ linkage names
# ---------------------------------------------------------------------------
def _sym(lib, name, argtypes):
    fn = getattr(lib, name)
    fn.restype = None
    fn.argtypes = argtypes
    return fn


@pytest.mark.parametrize("prec", ["f", "d"])
def test_dropin_symbols(native_built, prec):
    from cunfft_adjoint_gb300 import _lib
    P, I = ctypes.c_void_p, ctypes.c_int
    lib = _lib.dropin(prec)
    dt = np.float32 if prec == "f" else np.float64
    c = "f" if prec == "f" else "d"
    cplx = "P6float2" if prec == "f" else "P7double2"
    case = [g for g in PLAIN if g["x"].dtype == dt and g["name"].split("_")[1].startswith("n")][0]
    n, ng = len(case["x"]), int(case["ng"])
    gen = _sym(lib, "_Z26generate_filter_propertiesPK%siiPP17filter_propertiesS3_" % c, [P, I, I, P, P])
    raw = _sym(lib, "_Z24cunfft_adjoint_raw_asyncPK%sS0_%siiPK17filter_propertiesP11CUstream_st" % (c, cplx),
               [P, P, P, I, I, P, P])
    free_fp = _sym(lib, "_Z22free_filter_propertiesP17filter_propertiesS0_", [P, P])
    x, y = _dev(case["x"]), _dev(case["y"])
    h, d = P(), P()
    gen(x.data_ptr(), n, ng, ctypes.byref(h), ctypes.byref(d))
    f_hat = torch.zeros(ng, dtype=_ctype(dt), device="cuda")
    raw(x.data_ptr(), y.data_ptr(), f_hat.data_ptr(), n, ng, d, None)
    torch.cuda.synchronize()
    assert rel_l2(f_hat.cpu().numpy(), case["F"]) < _tol(dt)
    free_fp(d, h)
    # host-array convenience call (returns the result, unlike the reference)
    conv = _sym(lib, "_Z14cunfft_adjointPK%sS0_PC%siij" % (c, c), [P, P, P, I, I, ctypes.c_uint])
    out = np.zeros(ng, np.complex64 if prec == "f" else np.complex128)
    xa, ya = np.ascontiguousarray(case["x"]), np.ascontiguousarray(case["y"])
    conv(xa.ctypes.data, ya.ctypes.data, out.ctypes.data, n, ng, 0)
    assert rel_l2(out, case["F"]) < _tol(dt)


# ---------------------------------------------------------------------------
# plans: init_plan + cunfft_adjoint_from_plan against the reference's own
# src/utils.cu:95-178 and src/cuna_kernel.cu:137-145 (tests/golden/host)
# ---------------------------------------------------------------------------
class _Plan(ctypes.Structure):
    """The reference's plan (inc/cuna_typedefs.h:118-149), 96 bytes."""
    _fields_ = [("x_data", ctypes.c_void_p), ("f_data", ctypes.c_void_p), ("f_hat", ctypes.c_void_p),
                ("f_hat_win", ctypes.c_void_p), ("g_f_hat", ctypes.c_void_p), ("g_f_hat_win", ctypes.c_void_p),
                ("g_x_data", ctypes.c_void_p), ("g_f_data", ctypes.c_void_p), ("flags", ctypes.c_uint),
                ("Ndata", ctypes.c_int), ("Ngrid", ctypes.c_int), ("filter_radius", ctypes.c_int),
                ("fprops_host", ctypes.c_void_p), ("fprops_device", ctypes.c_void_p)]


def _plan_cases():
    import glob
    import os
    from conftest import GOLDEN_DIR
    out = []
    for f in sorted(glob.glob(os.path.join(GOLDEN_DIR, "host", "plan_*.npz"))):
        d = dict(np.load(f))
        d["name"] = os.path.basename(f)[:-4]
        out.append(d)
    return out


@pytest.mark.parametrize("case", _plan_cases(), ids=lambda c: c["name"])
def test_plan_from_reference_fixture(native_built, case):
    """init_plan copies the host arrays in and builds the filter;
    cunfft_adjoint_from_plan grids, transforms and normalises, and copies
    f_hat (and f_hat_win with CALCULATE_WINDOW_FUNCTION) back to the plan's
    host arrays -- which the reference means to do but never does (its flag
    test is always false), so its results are read with copyResultsToCPU."""
    from cunfft_adjoint_gb300 import _lib
    assert ctypes.sizeof(_Plan) == 96
    x, y = case["x"], case["y"]
    prec = "f" if x.dtype == np.float32 else "d"
    c = prec
    lib = _lib.dropin(prec)
    P, I = ctypes.c_void_p, ctypes.c_int
    init = _sym(lib, "_Z9init_planP4planPK%sS2_iij" % c, [P, P, P, I, I, ctypes.c_uint])
    run = _sym(lib, "_Z24cunfft_adjoint_from_planP4plan", [P])
    free_plan = _sym(lib, "_Z9free_planP4plan", [P])
    libc = ctypes.CDLL(None)
    libc.malloc.restype = ctypes.c_void_p
    libc.malloc.argtypes = [ctypes.c_size_t]
    pp = libc.malloc(96)  # free_plan releases the plan itself, as the reference's does
    n, ng, flags = int(case["n"]), int(case["ng"]), int(case["flags"])
    xa, ya = np.ascontiguousarray(x), np.ascontiguousarray(y)
    init(pp, xa.ctypes.data, ya.ctypes.data, n, ng, flags)
    run(pp)
    p = _Plan.from_address(pp)
    assert (p.Ndata, p.Ngrid, p.flags) == (n, ng, flags)
    ct = np.complex64 if prec == "f" else np.complex128
    f_hat = np.ctypeslib.as_array((ctypes.c_byte * (ng * np.dtype(ct).itemsize)).from_address(p.f_hat)).view(ct)
    tol = _tol(x.dtype)
    assert rel_l2(f_hat.copy(), case["f_hat"]) < tol
    if "f_hat_win" in case:
        win = np.ctypeslib.as_array((ctypes.c_byte * (ng * np.dtype(ct).itemsize)).from_address(p.f_hat_win)).view(ct)
        assert rel_l2(win.copy(), case["f_hat_win"]) < tol
    free_plan(pp)
