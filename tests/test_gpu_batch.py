"""GPU tests of the batched forms: bootstrap resampling in accurate mode
(cuna2_adjoint_bootstrap) and uneven batches of series (cuna2_batch_*),
against the FP64 direct NDFT of the oracle.  Bar: 1e-5 relative L2 (float)."""
import numpy as np
import pytest
import torch

from conftest import rel_l2

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def nfft(native_built):
    from cunfft_adjoint_gb300 import nfft as N
    return N


@pytest.mark.parametrize("n,nf,R,m,nbs", [(3000, 4096, 2, 8, 4), (20000, 65536, 2, 8, 3), (5000, 16384, 2, 8, 2),
                                           (5000, 32768, 2, 8, 3),
                                           (4000, 16384, 4, 12, 2)])
def test_bootstrap_resamples_vs_ndft(nfft, oracle_lib, n, nf, R, m, nbs):
    """Resample b uses samples d = xorshift32(wang_hash(seed + b*n + i)) % n
    (the reference's draw stream) at their own times: one-CTA plans (grids
    of up to 32,768 cells) and tiled plans (65,536 and 131,072 cells), m = 8
    and 12."""
    rng = np.random.default_rng(n)
    t = rng.uniform(0, 100.0, n)
    y = (np.sin(2 * np.pi * t / 2.1) + rng.normal(0, 0.3, n)).astype(np.float32)
    seed = 1234
    plan = nfft.AdjointNFFT(nf, R, m, torch.float32)
    F = plan.bootstrap(torch.as_tensor(t, device="cuda"), torch.as_tensor(y, device="cuda"), nbs, seed, 0.0, 100.0)
    torch.cuda.synchronize()
    F = F.cpu().numpy().astype(np.complex128)
    draws = oracle_lib.bootstrap_draws(seed, n, nbs).reshape(nbs, n)
    k = np.arange(-nf // 2, nf // 2)
    sel = k if nf <= 4096 else np.sort(rng.choice(k, 256, replace=False))
    for b in range(nbs):
        d = draws[b]
        D = oracle_lib.ndft(t[d], y[d].astype(np.float64), 0.0, 100.0, sel)
        assert rel_l2(F[b, sel + nf // 2], D) < 1e-5, b


def _batch_case(rng, ns, nmin, nmax, nf_cap):
    n = np.exp(rng.uniform(np.log(nmin), np.log(nmax), ns)).astype(np.int64)
    nf = np.minimum(2 ** np.ceil(np.log2(4 * n)).astype(np.int64), nf_cap)
    T = np.exp(rng.uniform(np.log(10), np.log(3000), ns))
    ts, ys = [], []
    for i in range(ns):
        t = rng.uniform(0, T[i], n[i])
        y = rng.normal(0, 1, n[i]) + 0.5 * np.sin(2 * np.pi * t / rng.uniform(0.5, 50))
        ts.append(t)
        ys.append(y.astype(np.float32))
    return n, nf, T, ts, ys


@pytest.mark.parametrize("graph", [False, True])
def test_uneven_batch_vs_ndft(nfft, oracle_lib, graph):
    rng = np.random.default_rng(11)
    n, nf, T, ts, ys = _batch_case(rng, 24, 60, 30000, 1 << 16)
    plan = nfft.BatchAdjointNFFT(n, nf, 2, 8, np.zeros(len(n)), T, torch.float32, graph=graph)
    td = torch.as_tensor(np.concatenate(ts), device="cuda")
    yd = torch.as_tensor(np.concatenate(ys), device="cuda")
    F = plan(td, yd)
    F2 = plan(td, yd)
    torch.cuda.synchronize()
    Fs = [f.cpu().numpy().astype(np.complex128) for f in plan.split(F)]
    assert torch.equal(F, F2) or rel_l2(F2.cpu().numpy(), F.cpu().numpy()) < 1e-6
    assert any(R * f > 32768 for R, f in zip([2] * len(nf), nf)) and any(2 * f <= 32768 for f in nf)
    for i in range(len(n)):
        k = np.arange(-nf[i] // 2, nf[i] // 2)
        sel = k if nf[i] <= 2048 else np.sort(rng.choice(k, 128, replace=False))
        D = oracle_lib.ndft(ts[i], ys[i].astype(np.float64), 0.0, T[i], sel)
        assert rel_l2(Fs[i][sel + nf[i] // 2], D) < 1e-5, (i, n[i], nf[i])


def test_uneven_batch_matches_single_plans(nfft):
    """The batched execution equals the per-series plans (same kernels)."""
    rng = np.random.default_rng(12)
    n, nf, T, ts, ys = _batch_case(rng, 6, 1000, 40000, 1 << 16)
    plan = nfft.BatchAdjointNFFT(n, nf, 2, 8, np.zeros(len(n)), T, torch.float32)
    F = plan(torch.as_tensor(np.concatenate(ts), device="cuda"), torch.as_tensor(np.concatenate(ys), device="cuda"))
    for i, Fi in enumerate(plan.split(F)):
        single = nfft.AdjointNFFT(int(nf[i]), 2, 8, torch.float32)
        Si = single(torch.as_tensor(ts[i], device="cuda"), torch.as_tensor(ys[i], device="cuda"), 0.0, T[i])
        torch.cuda.synchronize()
        assert rel_l2(Fi.cpu().numpy(), Si.cpu().numpy()) < 1e-6, i


def test_large_batch_multi_block_scan_and_classes(nfft, oracle_lib):
    """A batch whose large series need more than 8192 tiles (the multi-CTA
    tile scan) spread over four FFT size classes, against the NDFT."""
    rng = np.random.default_rng(23)
    nser = 200
    nf = np.array([1 << int(v) for v in rng.integers(15, 19, nser)], dtype=np.int64)
    n = rng.integers(500, 3000, nser).astype(np.int64)
    T = np.exp(rng.uniform(np.log(10), np.log(3000), nser))
    ts = [rng.uniform(0, T[i], n[i]) for i in range(nser)]
    ys = [rng.normal(0, 1, n[i]).astype(np.float32) for i in range(nser)]
    plan = nfft.BatchAdjointNFFT(n, nf, 2, 8, np.zeros(nser), T, torch.float32)
    F = plan(torch.as_tensor(np.concatenate(ts), device="cuda"), torch.as_tensor(np.concatenate(ys), device="cuda"))
    parts = plan.split(F)
    for i in rng.choice(nser, 8, replace=False):
        k = np.sort(rng.choice(np.arange(-nf[i] // 2, nf[i] // 2), 64, replace=False))
        D = oracle_lib.ndft(ts[i], ys[i].astype(np.float64), 0.0, T[i], k)
        assert rel_l2(parts[i].cpu().numpy()[k + nf[i] // 2], D) < 1e-5, i


def test_batch_with_empty_and_tiny_series(nfft, oracle_lib):
    """Series of 0, 1 and 2 samples (small and large grids) inside a batch:
    empty series give zero spectra, the others the NDFT."""
    rng = np.random.default_rng(31)
    n = np.array([0, 1, 2, 5000, 0, 1, 30000, 3], dtype=np.int64)
    nf = np.array([1024, 4096, 1 << 16, 1 << 14, 1 << 17, 1 << 16, 1 << 17, 256], dtype=np.int64)
    T = rng.uniform(10, 100, len(n))
    ts = [rng.uniform(0, T[i], n[i]) for i in range(len(n))]
    ys = [rng.normal(0, 1, n[i]).astype(np.float32) for i in range(len(n))]
    plan = nfft.BatchAdjointNFFT(n, nf, 2, 8, np.zeros(len(n)), T, torch.float32)
    F = plan(torch.as_tensor(np.concatenate(ts), device="cuda"), torch.as_tensor(np.concatenate(ys), device="cuda"))
    parts = [p.cpu().numpy() for p in plan.split(F)]
    for i in range(len(n)):
        if n[i] == 0:
            assert not np.any(parts[i]), i
            continue
        k = np.arange(-nf[i] // 2, nf[i] // 2)[:: max(1, nf[i] // 256)]
        D = oracle_lib.ndft(ts[i], ys[i].astype(np.float64), 0.0, T[i], k)
        assert rel_l2(parts[i][k + nf[i] // 2], D) < 1e-5, i


@pytest.mark.parametrize("dtype", [torch.float32, torch.float64])
def test_batch_schedules_and_autotune(nfft, oracle_lib, dtype):
    """Every schedule of a batched plan (tiles of 1024 to 8192 cells in
    fixed-point form, 1024 to 4096 in gather form) gives each series' NDFT spectrum, the
    schedules agree with each other to rounding, and the batch autotuner
    keeps one of them."""
    from cunfft_adjoint_gb300 import _lib
    rng = np.random.default_rng(29)
    n, nf, T, ts, ys = _batch_case(rng, 20, 2000, 60000, 1 << 17)
    yd_np = np.concatenate(ys).astype(np.float32 if dtype == torch.float32 else np.float64)
    plan = nfft.BatchAdjointNFFT(n, nf, 2, 8, np.zeros(len(n)), T, dtype)
    td = torch.as_tensor(np.concatenate(ts), device="cuda")
    yd = torch.as_tensor(yd_np, device="cuda")
    assert plan.schedule == (12, _lib.GRID_FIXED)
    offs = np.concatenate([[0], np.cumsum(n)])
    big = [i for i in range(len(n)) if nf[i] * 2 > (1 << 15)]
    outs = {}
    for gm in (_lib.GRID_FIXED, _lib.GRID_GATHER):
        for lt in ((10, 11, 12, 13) if gm == _lib.GRID_FIXED else (10, 11, 12)):
            plan.set_schedule(lt, gm)
            assert plan.schedule == (lt, gm)
            F = plan.split(plan(td, yd).cpu().numpy().astype(np.complex128))
            for i in big[:3]:
                k = np.arange(-nf[i] // 2, nf[i] // 2)
                sel = np.sort(rng.choice(k, 128, replace=False))
                D = oracle_lib.ndft(ts[i], yd_np[offs[i]:offs[i + 1]].astype(np.float64), 0.0, T[i], sel)
                assert rel_l2(F[i][sel + nf[i] // 2], D) < (1e-5 if dtype == torch.float32 else 5e-8), (lt, gm, i)
            outs[(lt, gm)] = np.concatenate(F)
    ref = outs[(12, _lib.GRID_FIXED)]
    for key, F in outs.items():
        assert rel_l2(F, ref) < (2e-6 if dtype == torch.float32 else 1e-13), key
    with pytest.raises(_lib.CunaError):
        plan.set_schedule(9, _lib.GRID_GATHER)
    with pytest.raises(_lib.CunaError):
        plan.set_schedule(11, _lib.GRID_SCATTER)
    with pytest.raises(_lib.CunaError):
        plan.set_schedule(13, _lib.GRID_GATHER)
    with pytest.raises(_lib.CunaError):
        plan.set_schedule(14, _lib.GRID_FIXED)
    lt, gm, ms = plan.autotune(td, yd, reps=2)
    assert (lt, gm) in outs and ms > 0
    assert rel_l2(plan(td, yd).cpu().numpy(), ref) < (2e-6 if dtype == torch.float32 else 1e-13)


@pytest.mark.parametrize("dtype,tol", [(torch.float32, 1e-5), (torch.float64, 1e-9)])
def test_batch_plan_for_tolerance(nfft, oracle_lib, dtype, tol):
    """cuna2_batch_plan_create_auto picks (R, m) per size class whose
    Gaussian error bound meets the target and a gridding schedule by the
    batch autotuner; the chosen plan's spectra meet the target against the
    FP64 NDFT."""
    rng = np.random.default_rng(31)
    n, nf, T, ts, ys = _batch_case(rng, 16, 100, 40000, 1 << 16)
    y_np = np.concatenate(ys).astype(np.float32 if dtype == torch.float32 else np.float64)
    td = torch.as_tensor(np.concatenate(ts), device="cuda")
    yd = torch.as_tensor(y_np, device="cuda")
    plan = nfft.BatchAdjointNFFT.for_tolerance(n, nf, tol, td, yd, np.zeros(len(n)), T, dtype)
    assert np.all(np.isin(plan.R, (2, 4, 8))) and np.all((plan.m >= 2) & (plan.m <= 16))
    assert np.all(np.exp(-np.pi * plan.m * np.sqrt(1 - 1 / plan.R)) <= tol)
    # one (R, m) per size class
    for v in np.unique(nf):
        assert len(set(zip(plan.R[nf == v], plan.m[nf == v]))) == 1
    F = plan.split(plan(td, yd).cpu().numpy().astype(np.complex128))
    offs = np.concatenate([[0], np.cumsum(n)])
    for i in range(0, len(n), 3):
        k = np.arange(-nf[i] // 2, nf[i] // 2)[:: max(1, nf[i] // 128)]
        D = oracle_lib.ndft(ts[i], y_np[offs[i]:offs[i + 1]].astype(np.float64), 0.0, T[i], k)
        # float plans reach their rounding (a few 1e-7) on top of the kernel error
        assert rel_l2(F[i][k + nf[i] // 2], D) < (1e-5 if dtype == torch.float32 else 5 * tol), i


def test_uneven_batch_full_size(nfft, oracle_lib):
    """The uneven workload at its full size (4096 series, N log-uniform in
    [100, 1e5], Nf = nextpow2(4N) capped at 2^18, R = 2, m = 8; about 61 M
    samples) under the batch's autotuned schedule: 12 series spread over the
    size range against the FP64 NDFT at 128 frequencies each, and linearity
    (the batch of 2y + 1 equals twice the batch of y plus the batch of ones)
    over every output."""
    rng = np.random.default_rng(4)
    ns = 4096
    n = np.exp(rng.uniform(np.log(100), np.log(1e5), ns)).astype(np.int64)
    nf = np.minimum(2 ** np.ceil(np.log2(4 * n)).astype(np.int64), 1 << 18)
    T = np.exp(rng.uniform(np.log(10), np.log(3000), ns))
    offs = np.concatenate([[0], np.cumsum(n)])
    t = np.concatenate([rng.uniform(0, T[i], n[i]) for i in range(ns)])
    y = rng.normal(0, 1, int(n.sum())).astype(np.float32)
    plan = nfft.BatchAdjointNFFT(n, nf, 2, 8, np.zeros(ns), T, torch.float32)
    td, yd = torch.as_tensor(t, device="cuda"), torch.as_tensor(y, device="cuda")
    plan.autotune(td, yd, reps=1)
    F = plan(td, yd).clone()
    order = np.argsort(n)
    pick = order[np.linspace(0, ns - 1, 12).astype(int)]
    parts = plan.split(F)
    for i in pick:
        k = np.sort(rng.choice(np.arange(-nf[i] // 2, nf[i] // 2), 128, replace=False))
        D = oracle_lib.ndft(t[offs[i]:offs[i + 1]], y[offs[i]:offs[i + 1]].astype(np.float64), 0.0, T[i], k)
        assert rel_l2(parts[i].cpu().numpy()[k + nf[i] // 2], D) < 1e-5, (i, n[i])
    G = plan(td, 2 * yd + 1).clone()
    G -= 2 * F
    G -= plan(td, torch.ones_like(yd))
    # G now holds the linearity residual; relative to the batch of 2y + 1
    res = float(torch.linalg.vector_norm(G)) / float(torch.linalg.vector_norm(plan(td, 2 * yd + 1)))
    assert res < 1e-5, res


def test_bootstrap_full_size(nfft, oracle_lib):
    """The bootstrap workload at its full size (N = 5000, 1024 resamples,
    Nf = 32768, R = 2, m = 8) under graph replay: 8 resamples spread over the
    batch against the FP64 NDFT of the resampled series at 256 frequencies,
    and every resample's spectrum equal to the single-resample bootstrap
    computed on its own (the same draws)."""
    rng = np.random.default_rng(3)
    n, nbs, nf, seed = 5000, 1024, 32768, 77
    t = rng.uniform(0, 100.0, n)
    y = (np.sin(2 * np.pi * t / 2.1) + rng.normal(0, 0.3, n)).astype(np.float32)
    td, yd = torch.as_tensor(t, device="cuda"), torch.as_tensor(y, device="cuda")
    plan = nfft.AdjointNFFT(nf, 2, 8, torch.float32)
    plan.set_graph(True)
    F = plan.bootstrap(td, yd, nbs, seed, 0.0, 100.0).cpu().numpy()
    draws = oracle_lib.bootstrap_draws_all(seed, n, nbs)
    k = np.sort(rng.choice(np.arange(-nf // 2, nf // 2), 256, replace=False))
    for b in np.linspace(0, nbs - 1, 8).astype(int):
        d = draws[b]
        D = oracle_lib.ndft(t[d], y[d].astype(np.float64), 0.0, 100.0, k)
        assert rel_l2(F[b, k + nf // 2].astype(np.complex128), D) < 1e-5, b
    # resample b of a seed is resample 0 of the seed advanced by b * n draws
    one = nfft.AdjointNFFT(nf, 2, 8, torch.float32)
    for b in (1, 511, 1023):
        Fb = one.bootstrap(td, yd, 1, (seed + b * n) & 0xFFFFFFFF, 0.0, 100.0).cpu().numpy()
        assert rel_l2(Fb[0], F[b]) < 1e-6, b


@pytest.mark.parametrize("dtype", [torch.float32, torch.float64])
def test_batch_per_series_filter_widths(nfft, oracle_lib, dtype):
    """Series of one batch with their own (R, m) (2, 8), (4, 5), (8, 4), (4,
    12) and (2, 16) over small and large grids, under every gridding form:
    each series' spectrum matches the FP64 NDFT to ten times its own kernel
    error bound (at least 1e-5 float, 1e-10 double)."""
    from cunfft_adjoint_gb300 import _lib
    rng = np.random.default_rng(37)
    n, nf, T, ts, ys = _batch_case(rng, 20, 200, 40000, 1 << 16)
    R = np.array([2, 4, 8, 4, 2] * 4)
    m = np.array([8, 5, 4, 12, 16] * 4)
    y_np = np.concatenate(ys).astype(np.float32 if dtype == torch.float32 else np.float64)
    td = torch.as_tensor(np.concatenate(ts), device="cuda")
    yd = torch.as_tensor(y_np, device="cuda")
    plan = nfft.BatchAdjointNFFT(n, nf, R, m, np.zeros(len(n)), T, dtype)
    offs = np.concatenate([[0], np.cumsum(n)])
    for lt, gm in ((12, _lib.GRID_FIXED), (12, _lib.GRID_GATHER), (13, _lib.GRID_FIXED)):
        plan.set_schedule(lt, gm)
        F = plan.split(plan(td, yd).cpu().numpy().astype(np.complex128))
        for i in range(len(n)):
            k = np.arange(-nf[i] // 2, nf[i] // 2)[:: max(1, nf[i] // 128)]
            D = oracle_lib.ndft(ts[i], y_np[offs[i]:offs[i + 1]].astype(np.float64), 0.0, T[i], k)
            bound = np.exp(-np.pi * m[i] * np.sqrt(1 - 1 / R[i]))
            # double plans also carry ~1e-11 beyond the Gaussian bound at
            # m = 12, R = 4 (the single-series double tests allow 1e-9)
            tol = max(10 * bound, 1e-5 if dtype == torch.float32 else 1e-10)
            assert rel_l2(F[i][k + nf[i] // 2], D) < tol, (lt, gm, i, R[i], m[i])


def test_batch_per_series_widths_reject_bad_values(nfft):
    """cuna2_batch_plan_create_ex rejects a per-series R below 2, m outside
    [1, 16], and an R that does not make R nf / 2 a power of two; the
    failure names the series."""
    from cunfft_adjoint_gb300 import _lib
    n = np.array([100, 200, 300], dtype=np.int64)
    nf = np.array([1024, 2048, 4096], dtype=np.int64)
    for R, m in (([2, 1, 2], [8, 8, 8]), ([2, 2, 2], [8, 17, 8]), ([2, 2, 2], [8, 8, 0]), ([2, 3, 2], [8, 8, 8])):
        with pytest.raises(_lib.CunaError, match="series"):
            nfft.BatchAdjointNFFT(n, nf, np.array(R), np.array(m))
    plan = nfft.BatchAdjointNFFT(n, nf, np.array([2, 4, 8]), np.array([8, 5, 4]))
    R = np.zeros(3, np.int32)
    m = np.zeros(3, np.int32)
    _lib.check(_lib.core().cuna2_batch_get_filter(plan._h, R.ctypes.data, m.ctypes.data))
    assert list(R) == [2, 4, 8] and list(m) == [8, 5, 4]
