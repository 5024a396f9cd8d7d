"""GPU tests of accurate mode (cuna2_plan_* / cuna2_adjoint) against the FP64
direct NDFT and the oracle's double-precision restatement.

Bars: float32 plans <= 1e-5 relative L2 against the FP64 NDFT; float64
plans at the Gaussian kernel's own accuracy (about exp(-pi m sqrt(1-1/R))).
"""
import numpy as np
import pytest
import torch

from conftest import rel_l2

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def nfft(native_built):
    from cunfft_adjoint_gb300 import nfft as N
    return N


def _run(N, t, y, nf, R, m, dtype, t0, T):
    plan = N.AdjointNFFT(nf, R, m, dtype)
    td = torch.as_tensor(t, dtype=torch.float64, device="cuda")
    yd = torch.as_tensor(y, dtype=dtype, device="cuda")
    F = plan(td, yd, t0, T)
    torch.cuda.synchronize()
    return F.cpu().numpy().astype(np.complex128)


CASES = [
    # n, nf, R, m, dtype, tol vs NDFT     (grid ng = R nf; small path if ng <= 2^15 f32 / 2^14 f64)
    (2000, 1024, 2, 8, torch.float32, 1e-5),
    (10000, 16384, 2, 8, torch.float32, 1e-5),         # cfg1 shape, fused single-CTA path
    (3000, 2048, 4, 12, torch.float64, 1e-11),
    (200_000, 1 << 16, 2, 8, torch.float32, 1e-5),     # four-step path
    (100_000, 1 << 15, 4, 12, torch.float64, 1e-11),   # four-step, double
    (200_000, 1 << 18, 2, 10, torch.float32, 1e-5),    # cfg5 shape
]


@pytest.mark.parametrize("n,nf,R,m,dtype,tol", CASES)
def test_vs_ndft(nfft, oracle_lib, n, nf, R, m, dtype, tol):
    rng = np.random.default_rng(n + nf)
    t = np.sort(rng.uniform(0, 500.0, n))
    y = rng.normal(0, 1, n) + 0.5 * np.sin(2 * np.pi * t / 3.7)
    y = y.astype(np.float32 if dtype == torch.float32 else np.float64)
    F = _run(nfft, t, y, nf, R, m, dtype, 0.0, 500.0)
    k = np.arange(-nf // 2, nf // 2)
    sel = k if nf <= 4096 else np.sort(rng.choice(k, 512, replace=False))
    D = oracle_lib.ndft(t, y.astype(np.float64), 0.0, 500.0, sel)
    assert rel_l2(F[sel + nf // 2], D) < tol
    # full spectrum against the oracle's restatement of the same algorithm
    O = oracle_lib.accurate_adjoint(t, y.astype(np.float64), 0.0, 500.0, nf, R, m)
    assert rel_l2(F, O) < max(tol, 1e-12)


def test_cfg2_full_size(nfft, oracle_lib):
    """N = 1e6 in 10 seasonal windows over 3650 d, Nf = 2^20, R = 4, m = 12,
    float32 (unsorted input), against the FP64 NDFT on 256 random bins."""
    rng = np.random.default_rng(2)
    n, nf = 1_000_000, 1 << 20
    win = rng.integers(0, 10, n)
    t = win * 365.0 + rng.uniform(0, 200.0, n)
    y = (np.sin(2 * np.pi * t / 0.7) + 0.3 * np.sin(2 * np.pi * t / 3.3) + 0.1 * np.sin(2 * np.pi * t / 41)
         + rng.normal(0, 1, n))
    F = _run(nfft, t, y.astype(np.float32), nf, 4, 12, torch.float32, 0.0, 3650.0)
    k = np.sort(rng.choice(np.arange(-nf // 2, nf // 2), 256, replace=False))
    D = oracle_lib.ndft(t, y.astype(np.float32).astype(np.float64), 0.0, 3650.0, k)
    assert rel_l2(F[k + nf // 2], D) < 1e-5


def test_long_baseline_phase(nfft, oracle_lib):
    """Julian-date times: t0 = 2.45e6 d; the fixed-point reduction keeps the
    phase exact where a float32 x would lose it entirely."""
    rng = np.random.default_rng(5)
    n, nf = 20000, 1 << 14
    t = 2450000.0 + np.sort(rng.uniform(0, 3000.0, n))
    y = rng.normal(0, 1, n).astype(np.float32)
    F = _run(nfft, t, y, nf, 2, 8, torch.float32, 2450000.0, 3000.0)
    k = np.arange(-nf // 2, nf // 2, 37)
    D = oracle_lib.ndft(t, y.astype(np.float64), 2450000.0, 3000.0, k)
    assert rel_l2(F[k + nf // 2], D) < 1e-5


def test_periodic_wrap(nfft):
    """Shifting every time by a multiple of T leaves F unchanged; samples
    outside [t0, t0 + T) wrap."""
    rng = np.random.default_rng(6)
    n, nf = 5000, 4096
    t = rng.uniform(0, 10.0, n)
    y = rng.normal(0, 1, n).astype(np.float32)
    A = _run(nfft, t, y, nf, 2, 8, torch.float32, 0.0, 10.0)
    B = _run(nfft, t + 30.0, y, nf, 2, 8, torch.float32, 0.0, 10.0)
    C = _run(nfft, t - 20.0, y, nf, 2, 8, torch.float32, 0.0, 10.0)
    assert rel_l2(B, A) < 1e-6 and rel_l2(C, A) < 1e-6


def test_linearity_and_hermitian(nfft):
    rng = np.random.default_rng(7)
    n, nf = 300_000, 1 << 17
    t = rng.uniform(0, 100.0, n)
    y1 = rng.normal(0, 1, n).astype(np.float32)
    y2 = rng.normal(0, 1, n).astype(np.float32)
    F1 = _run(nfft, t, y1, nf, 2, 8, torch.float32, 0.0, 100.0)
    F2 = _run(nfft, t, y2, nf, 2, 8, torch.float32, 0.0, 100.0)
    F3 = _run(nfft, t, (2 * y1 - 3 * y2).astype(np.float32), nf, 2, 8, torch.float32, 0.0, 100.0)
    assert rel_l2(F3, 2 * F1 - 3 * F2) < 1e-5
    K = nf // 2
    assert rel_l2(F1[K - np.arange(1, K)], np.conj(F1[K + np.arange(1, K)])) < 1e-6


def test_empty_and_single(nfft):
    F = _run(nfft, np.zeros(0), np.zeros(0, np.float32), 1024, 2, 8, torch.float32, 0.0, 1.0)
    assert np.all(F == 0)
    F = _run(nfft, np.array([0.25]), np.array([1.0], np.float32), 1024, 2, 8, torch.float32, 0.0, 1.0)
    k = np.arange(-512, 512)
    np.testing.assert_allclose(F, np.exp(2j * np.pi * k * (0.25 - 0.5)), atol=2e-6)


def test_plan_errors(nfft):
    from cunfft_adjoint_gb300 import CunaError
    with pytest.raises(CunaError):
        nfft.AdjointNFFT(1000, 3, 8)   # R*nf/2 not a power of two
    with pytest.raises(CunaError):
        nfft.AdjointNFFT(1024, 2, 40)  # m out of range


SCHED_CASES = [
    # n, nf, R, m, dtype, tol vs NDFT      (four-step path: tiles in use)
    (150_000, 1 << 16, 2, 8, torch.float32, 1e-5),
    (60_000, 1 << 15, 4, 12, torch.float64, 1e-11),
]


@pytest.mark.parametrize("n,nf,R,m,dtype,tol", SCHED_CASES)
def test_every_schedule(nfft, oracle_lib, n, nf, R, m, dtype, tol):
    """Every gridding form at every admissible tile size, after either
    binning form, gives the NDFT's spectrum; all agree with each other to
    rounding."""
    from cunfft_adjoint_gb300 import _lib
    rng = np.random.default_rng(n)
    t = rng.uniform(0, 500.0, n)
    y = rng.normal(0, 1, n).astype(np.float32 if dtype == torch.float32 else np.float64)
    td = torch.as_tensor(t, device="cuda")
    yd = torch.as_tensor(y, dtype=dtype, device="cuda")
    plan = nfft.AdjointNFFT(nf, R, m, dtype)
    k = np.arange(-nf // 2, nf // 2)
    sel = np.sort(rng.choice(k, 256, replace=False))
    D = oracle_lib.ndft(t, y.astype(np.float64), 0.0, 500.0, sel)
    outs = {}
    for gm, lt, bn in [(g, l, b) for b in (_lib.BIN_GLOBAL, _lib.BIN_LOCAL)
                       for g in (_lib.GRID_GATHER, _lib.GRID_SCATTER, _lib.GRID_FIXED)
                       for l in (9, 10, 11, 12, 13)]:
        plan.binning = bn
        if gm == _lib.GRID_GATHER and lt == 13:
            with pytest.raises(_lib.CunaError):
                plan.set_schedule(lt, gm)
            continue
        plan.set_schedule(lt, gm)
        assert plan.schedule == (lt, gm) and plan.binning == bn
        F = plan(td, yd, 0.0, 500.0).cpu().numpy().astype(np.complex128)
        assert rel_l2(F[sel + nf // 2], D) < tol, (lt, gm, bn)
        outs[(lt, gm, bn)] = F
    ref = outs[(12, _lib.GRID_GATHER, _lib.BIN_GLOBAL)]
    for key, F in outs.items():
        assert rel_l2(F, ref) < (2e-6 if dtype == torch.float32 else 1e-13), key


def test_schedule_rejects_bad_values(nfft):
    from cunfft_adjoint_gb300 import _lib
    plan = nfft.AdjointNFFT(1 << 16, 2, 16, torch.float32)
    for lt, gm in ((4, _lib.GRID_SCATTER), (14, _lib.GRID_SCATTER), (12, 7), (1, _lib.GRID_GATHER)):
        with pytest.raises(_lib.CunaError):
            plan.set_schedule(lt, gm)
    assert plan.schedule == (11, _lib.GRID_GATHER)


@pytest.mark.parametrize("dtype", [torch.float32, torch.float64])
def test_schedules_with_slab_weights(nfft, oracle_lib, dtype):
    """Bootstrap and multi-channel transforms (per-slab weights) under both
    gridding forms match each other and the per-resample transforms."""
    from cunfft_adjoint_gb300 import _lib
    rng = np.random.default_rng(3)
    n, nf, R, m = 5000, 1 << 14, 4, 8
    t = rng.uniform(0, 100.0, n)
    y = rng.normal(0, 1, n)
    td = torch.as_tensor(t, device="cuda")
    yd = torch.as_tensor(y, dtype=dtype, device="cuda")
    Y = torch.stack([yd, yd * 0 + 1, yd * yd])
    plan = nfft.AdjointNFFT(nf, R, m, dtype)
    res = []
    for gm, bn in [(g, b) for g in (_lib.GRID_GATHER, _lib.GRID_SCATTER, _lib.GRID_FIXED)
                   for b in (_lib.BIN_GLOBAL, _lib.BIN_LOCAL)]:
        plan.binning = bn
        plan.set_schedule(11, gm)
        B = plan.bootstrap(td, yd, 40, 17, 0.0, 100.0).cpu().numpy()
        M = plan.multi(td, Y, 0.0, 100.0).cpu().numpy()
        res.append((B, M))
    tol = 2e-6 if dtype == torch.float32 else 1e-13
    for other in res[1:]:
        assert rel_l2(res[0][0], other[0]) < tol
        assert rel_l2(res[0][1], other[1]) < tol
    D = oracle_lib.ndft(t, np.ones(n), 0.0, 100.0, np.arange(-nf // 2, nf // 2)[::64])
    # m = 8, R = 4: Gaussian kernel accuracy about exp(-pi m sqrt(1 - 1/R)) = 3.5e-10
    assert rel_l2(res[1][1][1][::64], D) < (1e-5 if dtype == torch.float32 else 2e-9)


@pytest.mark.parametrize("dtype,n,nf", [(torch.float32, 300_000, 1 << 18), (torch.float64, 300_000, 1 << 18),
                                        (torch.float32, 10_000, 1 << 14), (torch.float64, 8_000, 1 << 13)])
def test_autotune(nfft, oracle_lib, dtype, n, nf):
    """Autotuned plans (large: tiles x forms x binning; small: also the
    single-CTA path) still give the NDFT's spectrum."""
    from cunfft_adjoint_gb300 import _lib
    rng = np.random.default_rng(11)
    t = rng.uniform(0, 1000.0, n)
    y = rng.normal(0, 1, n)
    td = torch.as_tensor(t, device="cuda")
    yd = torch.as_tensor(y, dtype=dtype, device="cuda")
    plan = nfft.AdjointNFFT(nf, 2, 8, dtype)
    lt, gm, ms = plan.autotune(td, yd, 0.0, 1000.0, reps=3)
    assert 9 <= lt <= 13 and gm in (_lib.GRID_GATHER, _lib.GRID_SCATTER, _lib.GRID_FIXED)
    assert ms > 0
    assert plan.schedule == (lt, gm)
    F = plan(td, yd, 0.0, 1000.0).cpu().numpy().astype(np.complex128)
    sel = np.sort(rng.choice(np.arange(-nf // 2, nf // 2), 128, replace=False))
    D = oracle_lib.ndft(t, y, 0.0, 1000.0, sel)
    # m = 8, R = 2: Gaussian kernel accuracy about exp(-pi m sqrt(1 - 1/R)) = 1.9e-8
    assert rel_l2(F[sel + nf // 2], D) < (1e-5 if dtype == torch.float32 else 5e-8)


@pytest.mark.parametrize("dtype", [torch.float32, torch.float64])
def test_fixed_point_grid_is_reproducible(nfft, dtype):
    """The fixed-point form sums integers, so repeated runs (different atomic
    orders) give bit-identical spectra; a non-finite value turns its tiles,
    and so the spectrum, into NaN as float accumulation would."""
    from cunfft_adjoint_gb300 import _lib
    rng = np.random.default_rng(21)
    n, nf = 400_000, 1 << 17
    t = torch.as_tensor(rng.uniform(0, 100.0, n), device="cuda")
    y = torch.as_tensor(rng.normal(0, 1, n), dtype=dtype, device="cuda")
    plan = nfft.AdjointNFFT(nf, 2, 8, dtype)
    plan.set_schedule(12, _lib.GRID_FIXED)
    F1 = plan(t, y, 0.0, 100.0).clone()
    F2 = plan(t, y, 0.0, 100.0).clone()
    assert torch.equal(F1, F2)
    y[123] = float("nan")
    F3 = plan(t, y, 0.0, 100.0)
    assert torch.isnan(F3.real).any()


@pytest.mark.parametrize("dtype", [torch.float32, torch.float64])
def test_fixed_point_single_read_tiles(nfft, oracle_lib, dtype):
    """Fixed-point tiles of one slab with at most 1024 (float) / 512 (double)
    records stage them, build the bucket histogram and bound |y| in one read;
    denser tiles and weighted slabs (multi-channel) take the chunked path.
    Sparse samples with one dense burst give tiles of both kinds; channel 0
    of a multi-channel transform with values [y, 2y] runs the chunked path on
    the same records, so it must reproduce the plain transform's bits.  In
    double a cluster of 5000 samples inside one cell puts more than 2048
    records in a bucket: the tiles there keep one 64-bit atomic per tap, the
    others split each tap into two 32-bit atomics.  (In float such a
    cluster coarsens its tile's 2^-30 quantum past the 1e-5 bar.)"""
    from cunfft_adjoint_gb300 import _lib
    rng = np.random.default_rng(41)
    nf, T = 1 << 17, 100.0
    t = np.concatenate([rng.uniform(0, T, 20_000), rng.uniform(40.0, 40.5, 6000)])
    if dtype == torch.float64:
        t = np.concatenate([t, rng.uniform(70.0, 70.0001, 5000)])
    y = rng.normal(0, 1, t.size)
    td = torch.as_tensor(t, device="cuda")
    yd = torch.as_tensor(y, dtype=dtype, device="cuda")
    plan = nfft.AdjointNFFT(nf, 2, 8, dtype)
    plan.set_schedule(12, _lib.GRID_FIXED)
    F = plan(td, yd, 0.0, T).clone()
    M = plan.multi(td, torch.stack([yd, 2 * yd]), 0.0, T)
    assert torch.equal(M[0], F)
    sel = np.sort(rng.choice(np.arange(-nf // 2, nf // 2), 128, replace=False))
    D = oracle_lib.ndft(t, yd.cpu().numpy().astype(np.float64), 0.0, T, sel)
    assert rel_l2(F.cpu().numpy().astype(np.complex128)[sel + nf // 2], D) < (1e-5 if dtype == torch.float32 else 5e-8)


def test_host_async_two_streams(nfft):
    """cuna2_adjoint_host_async from pinned host arrays, two plans on two
    streams in flight together, equals the device-array transform."""
    from cunfft_adjoint_gb300 import _lib
    rng = np.random.default_rng(41)
    n, nf, T = 100_000, 1 << 16, 100.0
    ts = [np.ascontiguousarray(rng.uniform(0, T, n)) for _ in range(4)]
    ys = [rng.normal(0, 1, n).astype(np.float32) for _ in range(4)]
    plans = [nfft.AdjointNFFT(nf, 2, 8, torch.float32) for _ in range(2)]
    streams = [torch.cuda.Stream(), torch.cuda.Stream()]
    th = [torch.as_tensor(t).pin_memory() for t in ts]
    yh = [torch.as_tensor(y).pin_memory() for y in ys]
    Fh = [torch.empty(nf, dtype=torch.complex64).pin_memory() for _ in range(4)]
    L = _lib.core()
    for s in range(4):
        k = s % 2
        _lib.check(L.cuna2_adjoint_host_async(plans[k]._h, th[s].data_ptr(), yh[s].data_ptr(), Fh[s].data_ptr(),
                                              n, 0.0, T, streams[k].cuda_stream))
    torch.cuda.synchronize()
    for s in range(4):
        ref = plans[0](torch.as_tensor(ts[s], device="cuda"), torch.as_tensor(ys[s], device="cuda"), 0.0, T)
        assert rel_l2(Fh[s].numpy(), ref.cpu().numpy()) < 1e-6


def test_reserved_binning_many_blocks(nfft, oracle_lib):
    """10,000,001 unsorted samples on 2048 tiles: the two-launch reserved
    binning runs each block over several sub-chunks of 4096 samples and a
    partial one, with a ragged last block; the
    spectrum equals the one binned by the three-launch form (8192 tiles,
    more than the fused scan takes) and the NDFT."""
    from cunfft_adjoint_gb300 import _lib
    rng = np.random.default_rng(77)
    n, nf, T = 10_000_001, 1 << 20, 1000.0
    t = rng.uniform(0, T, n)
    y = rng.normal(0, 1, n).astype(np.float32)
    td = torch.as_tensor(t, device="cuda")
    yd = torch.as_tensor(y, device="cuda")
    plan = nfft.AdjointNFFT(nf, 4, 12, torch.float32)
    plan.binning = _lib.BIN_GLOBAL
    plan.set_schedule(11, _lib.GRID_GATHER)
    F1 = plan(td, yd, 0.0, T).cpu().numpy().astype(np.complex128)
    plan.set_schedule(9, _lib.GRID_GATHER)
    F2 = plan(td, yd, 0.0, T).cpu().numpy().astype(np.complex128)
    assert rel_l2(F1, F2) < 2e-6
    k = np.sort(rng.choice(np.arange(-nf // 2, nf // 2), 32, replace=False))
    D = oracle_lib.ndft(t, y.astype(np.float64), 0.0, T, k)
    assert rel_l2(F1[k + nf // 2], D) < 1e-5


@pytest.mark.parametrize("dtype,nf,R,tol", [(torch.float32, 1 << 24, 4, 1e-5), (torch.float64, 1 << 22, 4, 1e-9)])
def test_largest_plans(nfft, oracle_lib, dtype, nf, R, tol):
    """The largest grids a plan accepts (2^25 packed points float, 2^23
    double) against the NDFT on 64 bins; one point more is refused."""
    rng = np.random.default_rng(5)
    n, T = 300_000, 1000.0
    t = rng.uniform(0, T, n)
    y = rng.normal(0, 1, n)
    plan = nfft.AdjointNFFT(nf, R, 12, dtype)
    F = plan(torch.as_tensor(t, device="cuda"), torch.as_tensor(y, dtype=dtype, device="cuda"), 0.0, T)
    k = np.sort(rng.choice(np.arange(-nf // 2, nf // 2), 64, replace=False))
    D = oracle_lib.ndft(t, y, 0.0, T, k)
    assert rel_l2(F.cpu().numpy()[k + nf // 2], D) < tol
    del F, plan
    torch.cuda.empty_cache()
    from cunfft_adjoint_gb300 import _lib
    with pytest.raises(_lib.CunaError):
        nfft.AdjointNFFT(2 * nf, R, 12, dtype)


@pytest.mark.parametrize("dtype,tol", [(torch.float32, 1e-5), (torch.float64, 1e-9)])
def test_plan_for_tolerance(nfft, oracle_lib, dtype, tol):
    """The filter-width chooser returns a plan whose kernel error estimate
    meets the target and whose spectrum meets it against the NDFT."""
    rng = np.random.default_rng(8)
    n, nf, T = 100_000, 1 << 16, 200.0
    t = rng.uniform(0, T, n)
    y = rng.normal(0, 1, n)
    td = torch.as_tensor(t, device="cuda")
    yd = torch.as_tensor(y, dtype=dtype, device="cuda")
    plan = nfft.AdjointNFFT.for_tolerance(nf, tol, td, yd, 0.0, T, dtype)
    assert plan.R in (2, 4, 8) and 2 <= plan.m <= 16
    assert np.exp(-np.pi * plan.m * np.sqrt(1 - 1 / plan.R)) <= max(tol, 1e-7)
    F = plan(td, yd, 0.0, T).cpu().numpy()
    k = np.sort(rng.choice(np.arange(-nf // 2, nf // 2), 128, replace=False))
    D = oracle_lib.ndft(t, y, 0.0, T, k)
    assert rel_l2(F[k + nf // 2], D) < tol


_SWITCH_SCRIPT = r"""
import sys, numpy as np, torch
sys.path.insert(0, sys.argv[1])
from cunfft_adjoint_gb300 import nfft as N, _lib
out = {}
cases = [(nf, R, torch.float32) for nf in (1 << 13, 1 << 15, 1 << 17, 1 << 19, 1 << 21, 1 << 23) for R in (2, 4)]
if sys.argv[3] == "all":
    cases += [(nf, R, torch.float64) for nf in (1 << 12, 1 << 15, 1 << 18, 1 << 21) for R in (2, 4)]
for nf, R, dt in cases:
    rng = np.random.default_rng(nf + R)
    t = torch.as_tensor(rng.uniform(0, 100.0, 50_000), device="cuda")
    y = torch.as_tensor(rng.normal(0, 1, 50_000), dtype=dt, device="cuda")
    plan = N.AdjointNFFT(nf, R, 8, dt)
    plan.set_schedule(12, _lib.GRID_FIXED)
    for rep in range(2):
        out["%d_%d_%s_%d" % (nf, R, str(dt)[-7:], rep)] = plan(t, y, 0.0, 100.0).cpu().numpy()
np.savez(sys.argv[2], **out)
print(_lib.core().cuna2_wait_timeouts())
"""


def _spectra_under(tmp_path, tag, env, which):
    import os
    import subprocess
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    script = tmp_path / "switch.py"
    script.write_text(_SWITCH_SCRIPT)
    out = subprocess.run([sys.executable, str(script), root, str(tmp_path / (tag + ".npz")), which],
                         env={**os.environ, **env}, capture_output=True, text=True, timeout=900)
    assert out.returncode == 0, out.stderr[-2000:]
    assert out.stdout.strip().splitlines()[-1] == "0"
    return np.load(tmp_path / (tag + ".npz"))


def test_float_float_passes_match_fp64(tmp_path):
    """Double plans run their four-step passes in float-float arithmetic
    (default) or in FP64 (CUNA2_F64_PASSES=1): the same fixed-point grids give
    spectra within 1e-13 relative L2 of each other at packed lengths 2^12 ..
    2^22; float plans are untouched (bit-identical)."""
    a = _spectra_under(tmp_path, "df", {"CUNA2_F64_PASSES": "0"}, "all")
    b = _spectra_under(tmp_path, "fp64", {"CUNA2_F64_PASSES": "1"}, "all")
    for key in a.files:
        if "float32" in key:
            assert np.array_equal(a[key], b[key]), key
        else:
            assert rel_l2(a[key], b[key]) < 1e-13, key


def test_tma_column_pass_matches_plain(tmp_path):
    """The opt-in TMA column pass (CUNA2_TMA=1) stages its columns through
    tensor-map boxes (float packed lengths 2^13 .. 2^24 here); with
    fixed-point gridding (identical grids) its spectra are bit-identical to
    the default load/store column pass, and no bounded wait ran out."""
    a = _spectra_under(tmp_path, "tma", {"CUNA2_TMA": "1", "CUNA2_PDL": "0"}, "float")
    b = _spectra_under(tmp_path, "plain", {"CUNA2_TMA": "0", "CUNA2_PDL": "0"}, "float")
    for key in a.files:
        assert np.array_equal(a[key], b[key]), key


def test_dependent_launch_matches_serial(tmp_path):
    """Programmatic dependent launch (the default) lets each kernel of a
    transform start before its predecessor has finished; every float and
    double length with compile-time passes gives spectra bit-identical to
    fully serialised launches (CUNA2_PDL=0), twice in a row per plan (fixed-
    point gridding, so the grids are identical)."""
    a = _spectra_under(tmp_path, "pdl", {"CUNA2_PDL": "1"}, "all")
    b = _spectra_under(tmp_path, "serial", {"CUNA2_PDL": "0"}, "all")
    for key in a.files:
        assert np.array_equal(a[key], b[key]), key


def test_graph_replay_on_streams_matches_eager(nfft):
    """CUDA-graph replay (one graph per plan and input set, capturing the
    kernels' dependent-launch edges), three plans on three concurrent streams
    as the bench runs them, rotating input sets: every spectrum equals the
    eager transform of the same input bit for bit (fixed-point gridding)."""
    from cunfft_adjoint_gb300 import _lib
    L = _lib.core()
    rng = np.random.default_rng(3)
    n, nf, T = 200_000, 1 << 18, 100.0
    sets = [(torch.as_tensor(rng.uniform(0, T, n), device="cuda"),
             torch.as_tensor(rng.normal(0, 1, n), dtype=torch.float32, device="cuda")) for _ in range(3)]
    p0 = nfft.AdjointNFFT(nf, 4, 12, torch.float32)
    p0.set_schedule(11, _lib.GRID_FIXED)
    ref = [p0(t, y, 0.0, T).cpu().numpy() for t, y in sets]
    plans = [nfft.AdjointNFFT(nf, 4, 12, torch.float32) for _ in range(3)]
    streams = [torch.cuda.Stream() for _ in range(3)]
    outs = [torch.empty(nf, dtype=torch.complex64, device="cuda") for _ in range(3)]
    for p in plans:
        p.set_schedule(11, _lib.GRID_FIXED)
        _lib.check(L.cuna2_plan_set_graph(p._h, 1))
    torch.cuda.synchronize()
    for rnd in range(6):
        for k in range(3):
            t, y = sets[(k + rnd) % 3]
            _lib.check(L.cuna2_adjoint(plans[k]._h, t.data_ptr(), y.data_ptr(), outs[k].data_ptr(), n, 0.0, T,
                                       streams[k].cuda_stream))
        torch.cuda.synchronize()
        for k in range(3):
            assert np.array_equal(outs[k].cpu().numpy(), ref[(k + rnd) % 3]), (rnd, k)


_GATHER_SCRIPT = r"""
import sys
import numpy as np, torch
sys.path.insert(0, sys.argv[1])
from cunfft_adjoint_gb300 import nfft, _lib
rng = np.random.default_rng(21)
out = {}
for (n, nf, R, m) in ((200_000, 1 << 18, 4, 12), (150_000, 1 << 16, 2, 8), (40_000, 1 << 15, 2, 5)):
    t = torch.as_tensor(rng.uniform(0, 300.0, n), device="cuda")
    y = torch.as_tensor(rng.normal(0, 1, n).astype(np.float32), device="cuda")
    plan = nfft.AdjointNFFT(nf, R, m, torch.float32)
    plan.set_schedule(11, _lib.GRID_GATHER)
    out["F_%d_%d" % (R, m)] = plan(t, y, 0.0, 300.0).cpu().numpy()
    out["B_%d_%d" % (R, m)] = plan.bootstrap(t[:5000], y[:5000], 16, 3, 0.0, 300.0).cpu().numpy()
np.savez(sys.argv[2], **out)
"""


def test_unmasked_gather_matches_masked(tmp_path):
    """Float plans whose Gaussian is below 1e-8 of its peak beyond m cells
    (m = 12, R = 4 and m = 8, R = 2 here) grid each record into whole cell
    groups without the tap masks; the spectra agree with the masked form
    (CUNA2_GATHER_MASKS=1) to float rounding.  m = 5, R = 2 keeps the masks
    in both runs (only the order of records within a cell, which follows the
    shared-memory atomics, can differ)."""
    import os
    import subprocess
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    script = tmp_path / "gather.py"
    script.write_text(_GATHER_SCRIPT)
    res = {}
    for tag, env in (("masked", {"CUNA2_GATHER_MASKS": "1"}), ("free", {"CUNA2_GATHER_MASKS": "0"})):
        r = subprocess.run([sys.executable, str(script), root, str(tmp_path / (tag + ".npz"))],
                           env={**os.environ, **env}, capture_output=True, text=True, timeout=600)
        assert r.returncode == 0, r.stderr[-2000:]
        res[tag] = np.load(tmp_path / (tag + ".npz"))
    for key in res["masked"].files:
        assert rel_l2(res["free"][key], res["masked"][key]) < 1e-6, key


@pytest.mark.parametrize("dtype", [torch.float32, torch.float64])
def test_graph_replay_of_bootstrap_and_channels(nfft, dtype):
    """With graph replay on, a bootstrap graph is captured once per argument
    set and replayed with a new draw seed each call (the draw kernel's seed
    argument is updated in the instantiated graph); multi-channel calls are
    replayed too.  Fixed-point gridding makes the grids bit-reproducible, so
    replays must equal eager calls exactly, whatever order the seeds come in."""
    from cunfft_adjoint_gb300 import _lib
    rng = np.random.default_rng(13)
    n, nf = 6000, 1 << 14
    t = torch.as_tensor(rng.uniform(0, 50.0, n), device="cuda")
    y = torch.as_tensor(rng.normal(0, 1, n), dtype=dtype, device="cuda")
    Y = torch.stack([y, y * 0 + 1, y * y])
    eager = nfft.AdjointNFFT(nf, 2, 8, dtype)
    eager.set_schedule(11, _lib.GRID_FIXED)
    want = {s: eager.bootstrap(t, y, 24, s, 0.0, 50.0).cpu().numpy() for s in (5, 6, 7)}
    want_m = eager.multi(t, Y, 0.0, 50.0).cpu().numpy()
    plan = nfft.AdjointNFFT(nf, 2, 8, dtype)
    plan.set_schedule(11, _lib.GRID_FIXED)
    plan.set_graph(True)
    out = torch.empty((24, nf), dtype=plan.cdtype, device="cuda")
    for s in (5, 6, 5, 7, 7, 6):
        plan.bootstrap(t, y, 24, s, 0.0, 50.0, out=out)
        assert np.array_equal(out.cpu().numpy(), want[s]), s
    outm = torch.empty((3, nf), dtype=plan.cdtype, device="cuda")
    for _ in range(2):
        plan.multi(t, Y, 0.0, 50.0, out=outm)
        assert np.array_equal(outm.cpu().numpy(), want_m)


def test_profile_times_each_launch_on_the_device(nfft):
    """cuna2_plan_profile replays the transform as a graph with an event node
    after each launch: one positive duration per launch, F written, and the
    durations stable from call to call (no host enqueue gaps)."""
    import ctypes
    from cunfft_adjoint_gb300 import _lib
    rng = np.random.default_rng(17)
    n, nf = 400_000, 1 << 19
    t = torch.as_tensor(rng.uniform(0, 100.0, n), device="cuda")
    y = torch.as_tensor(rng.normal(0, 1, n).astype(np.float32), device="cuda")
    plan = nfft.AdjointNFFT(nf, 4, 12, torch.float32)
    F = torch.empty(nf, dtype=torch.complex64, device="cuda")
    ms = (ctypes.c_float * 16)()
    names = (ctypes.c_char_p * 16)()
    k = ctypes.c_int()
    runs = []
    for _ in range(5):
        F.zero_()
        _lib.check(_lib.core().cuna2_plan_profile(plan._h, t.data_ptr(), y.data_ptr(), F.data_ptr(), n, 0.0, 100.0,
                                                  None, ms, names, 16, ctypes.byref(k)))
        torch.cuda.synchronize()
        runs.append({names[i].decode(): ms[i] for i in range(k.value)})
    assert set(runs[0]) >= {"bin_count", "bin_scatter", "grid", "fft_colpass", "fft_rowpass", "event_gap"}
    for r in runs:
        assert all(v > 0 for key, v in r.items() if key != "event_gap") and r["event_gap"] >= 0
    # stable from call to call: of the four repeats, at most one (a clock or
    # neighbour event on a shared GPU) strays from the median by more than half
    med = {key: float(np.median([r[key] for r in runs])) for key in runs[0]}
    for key in runs[0]:
        off = [r[key] for r in runs[1:] if abs(r[key] - med[key]) >= 0.5 * med[key] + 0.002]
        assert len(off) <= 1, (key, [r[key] for r in runs], med[key])
    assert rel_l2(F.cpu().numpy(), plan(t, y, 0.0, 100.0).cpu().numpy()) < 1e-6


def test_time_grid_launch(nfft):
    """cuna2_plan_time_grid repeats the gridding launch of one transform back
    to back between two events: a positive mean time, and the transform's
    result unchanged by the repeats (the launch overwrites its grid)."""
    import ctypes
    from cunfft_adjoint_gb300 import _lib
    rng = np.random.default_rng(19)
    n, nf = 300_000, 1 << 19
    t = torch.as_tensor(rng.uniform(0, 100.0, n), device="cuda")
    y = torch.as_tensor(rng.normal(0, 1, n).astype(np.float32), device="cuda")
    plan = nfft.AdjointNFFT(nf, 4, 12, torch.float32)
    F = torch.empty(nf, dtype=torch.complex64, device="cuda")
    ms = ctypes.c_float()
    _lib.check(_lib.core().cuna2_plan_time_grid(plan._h, t.data_ptr(), y.data_ptr(), F.data_ptr(), n, 0.0, 100.0,
                                                20, None, ctypes.byref(ms)))
    assert 0 < ms.value < 1.0
    assert rel_l2(F.cpu().numpy(), plan(t, y, 0.0, 100.0).cpu().numpy()) < 1e-6
    small = nfft.AdjointNFFT(1024, 2, 8, torch.float32)
    Fs = torch.empty(1024, dtype=torch.complex64, device="cuda")
    assert _lib.core().cuna2_plan_time_grid(small._h, t.data_ptr(), y.data_ptr(), Fs.data_ptr(), 1000, 0.0, 100.0,
                                            5, None, ctypes.byref(ms)) == 3
