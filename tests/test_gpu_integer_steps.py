"""Bit-exact GPU checks of every integer step on the path, through the C-ABI.

The device's own values are read back by the cuna2_inspect_* entry points,
which run the same device functions as the transforms, and compared with the
oracle by exact equality:

* compat mode (src/gridding.cu:43-58,93-110, src/gaussian_filter.cu:213):
  the cell j, the filter origin u and the tap range [ms, me) of every
  sample, clamped (fast_gridding) and unclamped (fast_gridding_bootstrap);
  the bootstrap draws d = xorshift32(wang_hash(seed + i)) % n
  (src/gridding.cu:67-82,101); the tile of every record of the binning and
  the record's payload;
* accurate mode: the 64-bit fixed-point phase and cell of every sample, and
  the tile, cell, fractional cell, value and sample index of every record of
  a plan's binning, on both binning paths (reserved: up to 4096 tiles; scan
  and scatter: more).

Inputs: the plain 1e4-sample shape (ng = 32768), the large 1e6-sample
seasonal shape (ng = 2^22), the 1024 x 5000 bootstrap draws, and adversarial
values: x where (x + 1/2)(ng - 1) or ng x - R_f lies within a few ulps of an
integer, x = +-1/2 exactly and just outside, zero, infinities, NaN, huge
values, grids that are not powers of two; times at cell boundaries, at t0
and t0 + T, negative, subnormal and huge times, Julian-date baselines.
Within a tile the binning's records are compared as sets: their order
follows the scheduling of atomics and no result depends on it.
"""
import ctypes
from fractions import Fraction

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def L(native_built):
    from cunfft_adjoint_gb300 import _lib
    return _lib


def _dev(a):
    return torch.as_tensor(np.ascontiguousarray(a), device="cuda")


def _ptr(t):
    return None if t is None else t.data_ptr()


def _stream():
    return torch.cuda.current_stream().cuda_stream or None


# ---------------------------------------------------------------------------
# inputs
# ---------------------------------------------------------------------------

def plain_x(seed=0, n=10_000):
    rng = np.random.default_rng(seed)
    t = np.sort(rng.uniform(0, 1, n))
    return (t - t[0]) / (t[-1] - t[0]) - 0.5


def large_t(seed=2, n=1_000_000):
    rng = np.random.default_rng(seed)
    win = rng.integers(0, 10, n)
    return win * 365.0 + rng.uniform(0, 200.0, n)


def large_x(seed=2, n=1_000_000):
    t = large_t(seed, n)
    return t / 3650.0 - 0.5


def _nudge(v, dt, k):
    """v moved by k ulps in precision dt."""
    v = np.asarray(v, dt)
    inf = np.array(np.inf, dt)
    for _ in range(abs(k)):
        v = np.nextafter(v, inf if k > 0 else -inf)
    return v


def adversarial_x(ng, dt, rf, seed=5, per=64):
    """x where (x + 1/2)(ng - 1) and ng x - R_f sit on or next to integers,
    plus the edges and the non-finite values."""
    rng = np.random.default_rng(seed)
    out = []
    ks = np.concatenate([[0, 1, 2, ng // 2, ng - 2, ng - 1, ng], rng.integers(0, ng, per)])
    for k in ks:
        base_j = np.asarray(k / (ng - 1) - 0.5, dt)       # (x + 1/2)(ng - 1) = k
        base_u = np.asarray((k + rf) / ng, dt)             # ng x - rf = k
        base_v = np.asarray((k + rf) / ng - 0.5, dt)       # ng x - rf = k - ng/2
        for b in (base_j, base_u, base_v):
            for d in (-3, -2, -1, 0, 1, 2, 3):
                out.append(_nudge(b, dt, d))
    half = np.asarray(0.5, dt)
    for d in range(-4, 5):
        out += [_nudge(half, dt, d), _nudge(-half, dt, d)]
    out += [np.asarray(v, dt) for v in (0.0, -0.0, 1e-30, -1e-30, 0.75, -0.75, 2.0, -2.0, 1e6, -1e6,
                                         3e9, -3e9, np.inf, -np.inf, np.nan)]
    return np.array(out, dt).ravel()


# ---------------------------------------------------------------------------
# compat: cell, origin, tap range
# ---------------------------------------------------------------------------

def _compat_taps_device(L, x, ng, clamp):
    dt = x.dtype
    n = len(x)
    xd = _dev(x)
    outs = [torch.empty(n, dtype=torch.int32, device="cuda") for _ in range(4)]
    fn = L.core().cuna2_inspect_compat_taps_f32 if dt == np.float32 else L.core().cuna2_inspect_compat_taps_f64
    L.check(fn(_ptr(xd), n, ng, 1 if clamp else 0, *[_ptr(o) for o in outs], _stream()))
    torch.cuda.synchronize()
    return [o.cpu().numpy() for o in outs]


def _check_taps(L, oracle_lib, x, ng, clamp):
    dt = x.dtype
    got = _compat_taps_device(L, x, ng, clamp)
    want = oracle_lib.compat_taps(x, ng, dt, clamp)
    for name, g, w in zip(("cell", "origin", "tap_lo", "tap_hi"), got, want):
        bad = np.flatnonzero(g != w)
        assert bad.size == 0, "%s differs at %d samples, first x=%r: device %d oracle %d" % (
            name, bad.size, x[bad[0]], g[bad[0]], w[bad[0]])
    return got


COMPAT_CASES = [
    ("plain", np.float32, 32768),
    ("plain", np.float64, 32768),
    ("large", np.float32, 1 << 22),
    ("large", np.float64, 1 << 22),
]


@pytest.mark.parametrize("shape,dt,ng", COMPAT_CASES, ids=lambda v: getattr(v, "__name__", str(v)))
@pytest.mark.parametrize("clamp", [True, False])
def test_compat_taps_workloads(L, oracle_lib, shape, dt, ng, clamp):
    x = (plain_x() if shape == "plain" else large_x()).astype(dt)
    j, u, ms, me = _check_taps(L, oracle_lib, x, ng, clamp)
    # in-range samples: the taps never leave the grid
    has = ms < me
    assert np.all(j[has] + ms[has] >= 0) and np.all(j[has] + me[has] <= ng)


@pytest.mark.parametrize("dt", [np.float32, np.float64], ids=["f32", "f64"])
@pytest.mark.parametrize("ng", [32768, 3000, 40000, 1 << 22, 7])
@pytest.mark.parametrize("clamp", [True, False])
def test_compat_taps_adversarial(L, oracle_lib, dt, ng, clamp):
    rf = 6 if dt == np.float32 else 12
    x = adversarial_x(ng, dt, rf)
    j, u, ms, me = _check_taps(L, oracle_lib, x, ng, clamp)
    has = ms < me
    assert np.all(j[has].astype(np.int64) + ms[has] >= 0)
    assert np.all(j[has].astype(np.int64) + me[has] <= ng)


def test_compat_cell_exactness_f32(L):
    """For float x with 1/8 <= |x| <= 1/2 the product (x + 1/2)(ng - 1) is
    exact in double (x + 1/2 needs at most 26 significant bits, ng - 1 at
    most 22), so j is the exact truncation: check it against rational
    arithmetic on the cell-boundary inputs."""
    ng = 1 << 22
    x = adversarial_x(ng, np.float32, 6)
    x = x[np.isfinite(x) & (np.abs(x) >= 0.125) & (np.abs(x) <= 0.5)]
    j = _compat_taps_device(L, x, ng, False)[0]
    for xi, ji in zip(x, j):
        exact = (Fraction(float(xi)) + Fraction(1, 2)) * (ng - 1)
        want = int(exact) if exact >= 0 else -int(-exact)  # truncation toward zero
        assert ji == want, (xi, ji, want)


# ---------------------------------------------------------------------------
# bootstrap draws
# ---------------------------------------------------------------------------

@pytest.mark.parametrize("n,nbs,seed", [(5000, 1024, 7), (1, 5, 3), (3, 1000, 0xFFFFFFF0), (65537, 33, 12345)])
def test_bootstrap_draws(L, oracle_lib, n, nbs, seed):
    d = torch.empty(n * nbs, dtype=torch.int32, device="cuda")
    L.check(L.core().cuna2_inspect_bootstrap_draws(n, nbs, seed, _ptr(d), _stream()))
    torch.cuda.synchronize()
    want = oracle_lib.bootstrap_draws_all(seed, n, nbs).ravel()
    assert np.array_equal(d.cpu().numpy(), want)


# ---------------------------------------------------------------------------
# compat binning
# ---------------------------------------------------------------------------

REC_F32 = np.dtype([("cell", "<i4"), ("a", "<u4"), ("b", "<u4"), ("p", "<i4")])
REC_F32_VAL = np.dtype([("cell", "<i4"), ("a", "<u4"), ("b", "<u4"), ("p", "<u4")])  # p: the value's bits
REC_F64 = np.dtype([("cell", "<i4"), ("p", "<i4"), ("a", "<u8"), ("b", "<u8"), ("v", "<u8")])


def _compat_bins_device(L, x, y, ng, boot):
    from cunfft_adjoint_gb300 import cuna
    dt = x.dtype
    n = len(x)
    xd, yd = _dev(x), _dev(y)
    fp = cuna.generate_filter_properties(xd, n, ng)
    ntiles = (ng + 4095) // 4096
    offs = torch.empty(ntiles + 1, dtype=torch.int32, device="cuda")
    maxr = 2 * n
    rdt = REC_F32 if dt == np.float32 else REC_F64
    recs = torch.empty(maxr * rdt.itemsize, dtype=torch.uint8, device="cuda")
    nrec = ctypes.c_int()
    fn = L.core().cuna2_inspect_compat_bins_f32 if dt == np.float32 else L.core().cuna2_inspect_compat_bins_f64
    L.check(fn(_ptr(xd), _ptr(yd), n, ng, fp.data_ptr(), 1 if boot else 0, _ptr(offs), _ptr(recs), maxr,
               ctypes.byref(nrec), _stream()))
    torch.cuda.synchronize()
    R = recs.cpu().numpy()[:nrec.value * rdt.itemsize].view(rdt)
    if dt == np.float32 and not boot:
        R = R.view(REC_F32_VAL)
    E1 = fp.E1[:n].cpu().numpy().view(np.uint32 if dt == np.float32 else np.uint64)
    E2 = fp.E2[:n].cpu().numpy().view(np.uint32 if dt == np.float32 else np.uint64)
    return offs.cpu().numpy(), R, E1, E2


def _expected_compat_records(oracle_lib, x, y, ng, boot, E1, E2):
    """Per tile, the sorted rows of the records the reference's gridding
    thread of each sample feeds into that tile."""
    dt = x.dtype
    j, u, ms, me = oracle_lib.compat_taps(x, ng, dt, clamp=not boot)
    t0, t1 = oracle_lib.compat_tiles(j, ms, me)
    ybits = np.ascontiguousarray(y, dt).view(np.uint32 if dt == np.float32 else np.uint64)
    idx = np.arange(len(x))
    rows = {}
    for tiles in (t0, np.where(t1 != t0, t1, -1)):
        sel = tiles >= 0
        for t, jj, i in zip(tiles[sel], j[sel], idx[sel]):
            key = (int(jj), int(i)) if boot else (int(jj), int(E1[i]), int(E2[i]), int(ybits[i]))
            rows.setdefault(int(t), []).append(key)
    return {t: sorted(v) for t, v in rows.items()}


def _device_compat_rows(R, offs, boot, dt):
    rows = {}
    for t in range(len(offs) - 1):
        seg = R[offs[t]:offs[t + 1]]
        if len(seg) == 0:
            continue
        if boot:
            key = list(zip(seg["cell"].tolist(), seg["p"].tolist()))
        elif dt == np.float32:
            key = list(zip(seg["cell"].tolist(), seg["a"].tolist(), seg["b"].tolist(), seg["p"].tolist()))
        else:
            key = list(zip(seg["cell"].tolist(), seg["a"].tolist(), seg["b"].tolist(), seg["v"].tolist()))
        rows[t] = sorted(key)
    return rows


@pytest.mark.parametrize("case", [
    ("plain", np.float32, 32768, False),
    ("plain", np.float64, 32768, False),
    ("large", np.float32, 1 << 22, False),
    ("boot", np.float32, 65536, True),
    ("boot", np.float64, 65536, True),
    ("adv", np.float32, 40000, False),
    ("adv", np.float32, 1 << 22, True),
    ("many_tiles", np.float32, 1 << 25, False),   # 8192 tiles: the scan + scatter path
], ids=lambda c: "%s-%s-%d" % (c[0], np.dtype(c[1]).name, c[2]))
def test_compat_binning(L, oracle_lib, case):
    shape, dt, ng, boot = case
    rng = np.random.default_rng(9)
    if shape == "plain":
        x = plain_x()
    elif shape == "large":
        x = large_x()
    elif shape == "boot":
        x = np.sort(rng.uniform(0, 100, 5000)) / 100 - 0.5
    elif shape == "many_tiles":
        x = rng.uniform(-0.5, 0.5, 100_000)
    else:
        x = adversarial_x(ng, dt, 6 if dt == np.float32 else 12)
        x = x[np.isfinite(x)]
    x = x.astype(dt)
    y = rng.normal(0, 1, len(x)).astype(dt)
    offs, R, E1, E2 = _compat_bins_device(L, x, y, ng, boot)
    assert offs[0] == 0 and np.all(np.diff(offs) >= 0) and offs[-1] == len(R)
    want = _expected_compat_records(oracle_lib, x, y, ng, boot, E1, E2)
    got = _device_compat_rows(R, offs, boot, dt)
    assert set(got) == set(want), "tiles with records differ"
    for t in want:
        assert got[t] == want[t], "tile %d: records differ" % t


# ---------------------------------------------------------------------------
# accurate: phases and cells
# ---------------------------------------------------------------------------

def _phases_device(L, t, t0, T, ng):
    n = len(t)
    td = _dev(np.asarray(t, np.float64))
    S = torch.empty(n, dtype=torch.int64, device="cuda")
    cell = torch.empty(n, dtype=torch.int32, device="cuda")
    L.check(L.core().cuna2_inspect_phases(_ptr(td), n, float(t0), float(T), int(ng), _ptr(S), _ptr(cell),
                                          _stream()))
    torch.cuda.synchronize()
    return S.cpu().numpy().view(np.uint64), cell.cpu().numpy()


def adversarial_t(t0, T, ng, seed=4):
    rng = np.random.default_rng(seed)
    ks = np.concatenate([[0, 1, ng // 2, ng - 1, ng], rng.integers(0, ng, 48)])
    out = []
    for k in ks:
        b = t0 + k * (T / ng)
        for d in range(-3, 4):
            out.append(_nudge(b, np.float64, d))
    for v in (t0, t0 + T, t0 - T, t0 + 2 * T, t0 - 0.5 * T, -t0, 0.0, -0.0, 5e-324, -5e-324, 1e-300,
              1e300, -1e300, t0 + 1e6 * T, t0 - 1e6 * T):
        out.append(np.float64(v))
    return np.array(out, np.float64).ravel()


PHASE_CASES = [
    ("large", 0.0, 3650.0, 1 << 22),
    ("julian", 2.45e6, 3650.0 * 1.0001, 1 << 22),
    ("adv", 0.0, 3650.0, 1 << 22),
    ("adv_julian", 2451545.0, 1234.5678, 1 << 19),
    ("adv_nonpow2", 17.25, 3.0, 3 * (1 << 20)),
    ("adv_unit", 0.0, 1.0, 1 << 16),
]


@pytest.mark.parametrize("case", PHASE_CASES, ids=lambda c: c[0])
def test_accurate_phases(L, oracle_lib, case):
    name, t0, T, ng = case
    if name == "large":
        t = large_t()
    elif name == "julian":
        t = t0 + large_t(seed=3, n=200_000)
    else:
        t = adversarial_t(t0, T, ng)
    S, cell = _phases_device(L, t, t0, T, ng)
    So, co, _, _ = oracle_lib.phases(t, t0, T, ng)
    bad = np.flatnonzero(S != So)
    assert bad.size == 0, "phase differs at %d samples, first t=%r" % (bad.size, t[bad[0]])
    assert np.array_equal(cell, co)
    assert np.all((cell >= 0) & (cell < ng))


# ---------------------------------------------------------------------------
# accurate: the plan's binning
# ---------------------------------------------------------------------------

def _plan_bins_device(L, plan, t, y, t0, T):
    n = len(t)
    td, yd = _dev(np.asarray(t, np.float64)), _dev(y)
    lt, _ = plan.schedule
    ntiles = (plan.ng + (1 << lt) - 1) >> lt
    offs = torch.empty(ntiles + 1, dtype=torch.int32, device="cuda")
    rdt = REC_F32 if y.dtype == np.float32 else REC_F64
    maxr = 2 * n
    recs = torch.empty(maxr * rdt.itemsize, dtype=torch.uint8, device="cuda")
    nrec = ctypes.c_int64()
    L.check(L.core().cuna2_plan_inspect_bins(plan._h, _ptr(td), _ptr(yd), n, float(t0), float(T), _ptr(offs),
                                             _ptr(recs), maxr, ctypes.byref(nrec), _stream()))
    torch.cuda.synchronize()
    return lt, offs.cpu().numpy(), recs.cpu().numpy()[:nrec.value * rdt.itemsize].view(rdt)


@pytest.mark.parametrize("case", [
    ("large", np.float32, 1 << 20, 4, 12, None),       # 2048 tiles: reserved binning
    ("large", np.float64, 1 << 20, 4, 12, None),
    ("large", np.float32, 1 << 20, 4, 12, 9),          # 8192 tiles: scan + scatter
    ("julian", np.float32, 1 << 18, 2, 10, None),
    ("adv", np.float32, 1 << 17, 2, 8, None),
    ("adv", np.float64, 1 << 17, 2, 8, None),
], ids=lambda c: "%s-%s-nf%d-R%d-m%d-lt%s" % (c[0], np.dtype(c[1]).name, c[2], c[3], c[4], c[5]))
def test_accurate_binning(L, oracle_lib, case):
    from cunfft_adjoint_gb300 import nfft
    name, dt, nf, R, m, lt = case
    tdt = torch.float32 if dt == np.float32 else torch.float64
    plan = nfft.AdjointNFFT(nf, R, m, tdt)
    if lt is not None:
        plan.set_schedule(lt, plan.schedule[1])
    ng = plan.ng
    if name == "large":
        t0, T, t = 0.0, 3650.0, large_t(seed=6, n=1_000_000 if dt == np.float32 else 300_000)
    elif name == "julian":
        t0, T = 2.45e6, 500.0
        t = t0 + np.sort(np.random.default_rng(8).uniform(0, 500, 200_000))
    else:
        t0, T = 11.0, 250.0
        t = adversarial_t(t0, T, ng)
    y = np.random.default_rng(1).normal(0, 1, len(t)).astype(dt)
    log_tile, offs, Rr = _plan_bins_device(L, plan, t, y, t0, T)
    assert offs[0] == 0 and np.all(np.diff(offs) >= 0) and offs[-1] == len(Rr)
    S, cell, f24, f53 = oracle_lib.phases(t, t0, T, ng)
    ta, tb = oracle_lib.accurate_tiles(cell, ng, m, log_tile)
    ybits = y.view(np.uint32 if dt == np.float32 else np.uint64)
    if dt == np.float32:
        fbits = (f24.astype(np.float32) * np.float32(2.0 ** -24)).view(np.uint32)
    else:
        fbits = (f53.astype(np.float64) * 2.0 ** -53).view(np.uint64)
    want = {}
    idx = np.arange(len(t))
    for tiles in (ta, np.where(tb != ta, tb, -1)):
        sel = tiles >= 0
        for tt, i in zip(tiles[sel], idx[sel]):
            want.setdefault(int(tt), []).append((int(cell[i]), int(fbits[i]), int(ybits[i]), int(i)))
    got = {}
    for tt in range(len(offs) - 1):
        seg = Rr[offs[tt]:offs[tt + 1]]
        if len(seg):
            got[tt] = sorted(zip(seg["cell"].tolist(), seg["a"].tolist(), seg["b"].tolist(), seg["p"].tolist()))
    assert set(got) == set(want)
    for tt in want:
        assert got[tt] == sorted(want[tt]), "tile %d: records differ" % tt


def test_inspect_rejects_untiled_plans(L):
    from cunfft_adjoint_gb300 import nfft
    plan = nfft.AdjointNFFT(1024, 2, 8, torch.float32)  # one-CTA plan: no binning
    t = _dev(np.linspace(0, 1, 100, endpoint=False))
    y = _dev(np.ones(100, np.float32))
    offs = torch.empty(2, dtype=torch.int32, device="cuda")
    nrec = ctypes.c_int64()
    s = L.core().cuna2_plan_inspect_bins(plan._h, _ptr(t), _ptr(y), 100, 0.0, 1.0, _ptr(offs), None, 0,
                                         ctypes.byref(nrec), _stream())
    assert s == 3  # CUNA2_ERROR_UNSUPPORTED
