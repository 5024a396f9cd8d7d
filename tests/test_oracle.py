"""CPU tests: the oracle against the golden vectors of the reference's own
sources (tests/golden, made by tests/golden/make_golden.py) and against the
FP64 direct NDFT."""
import numpy as np
import pytest

from conftest import golden_cases, rel_l2

PLAIN = golden_cases("plain")
BOOT = golden_cases("boot")


def _prec(case):
    return "f" if case["x"].dtype == np.float32 else "d"


def _pow2(ng):
    return ng & (ng - 1) == 0


@pytest.mark.parametrize("case", PLAIN + BOOT, ids=lambda c: c["name"])
def test_filter_properties_match_reference(oracle_lib, case):
    """b, normfac, filter_radius, E1, E2, E3 of generate_filter_properties
    (src/gaussian_filter.cu:104-164,204-228)."""
    O = oracle_lib
    b, nf, rf, E1, E2, E3 = O.compat_filter(case["x"], int(case["ng"]), _prec(case))
    assert b == case["b"] and nf == case["normfac"] and rf == int(case["rf"])
    np.testing.assert_array_equal(E3, case["E3"])
    if _pow2(int(case["ng"])):
        # ng*x is exact for a power-of-two grid, so contraction cannot differ
        np.testing.assert_array_equal(E1, case["E1"])
        np.testing.assert_array_equal(E2, case["E2"])
    else:
        # the oracle contracts ng*x - u into one FMA as nvcc does for the
        # reference GPU build; the CPU-built golden rounds twice
        assert np.max(np.abs(E1 / case["E1"] - 1)) < 2e-3
        assert np.max(np.abs(E2 / case["E2"] - 1)) < 2e-3


@pytest.mark.parametrize("case", PLAIN, ids=lambda c: c["name"])
def test_gridding_matches_reference(oracle_lib, case):
    O = oracle_lib
    ng = int(case["ng"])
    g = O.compat_grid(case["x"], case.get("y"), ng, _prec(case))
    ref = case["grid"]
    if "f_hat0" in case:
        g = g + case["f_hat0"].real.astype(np.float64)
        np.testing.assert_array_equal(ref.imag, case["f_hat0"].imag)
    else:
        assert np.all(ref.imag == 0)  # only .x is accumulated (src/gridding.cu:62)
    tol = 1e-6 if _prec(case) == "f" else 1e-14
    if not _pow2(ng):
        tol = 5e-5
    assert rel_l2(g, ref.real) < tol


@pytest.mark.parametrize("case", PLAIN, ids=lambda c: c["name"])
def test_adjoint_matches_reference(oracle_lib, case):
    O = oracle_lib
    ng = int(case["ng"])
    F = O.compat_adjoint(case["x"], case.get("y"), ng, _prec(case), case.get("f_hat0"))
    tol = 1e-6 if _prec(case) == "f" else 1e-13
    if not _pow2(ng):
        tol = 5e-5
    assert rel_l2(F, case["F"]) < tol
    np.testing.assert_array_equal(case["F"], case["F_async"])


@pytest.mark.parametrize("case", BOOT, ids=lambda c: c["name"])
def test_bootstrap_matches_reference(oracle_lib, case):
    """Draw stream d = xorshift32(wang_hash(seed + i)) % n, position from
    x[i % n], slab (i / n) * ng (src/gridding.cu:67-117)."""
    O = oracle_lib
    ng, nbs, seed = int(case["ng"]), int(case["nbs"]), int(case["seed"])
    g = O.compat_grid_bootstrap(case["x"], case.get("y"), ng, nbs, seed, _prec(case))
    tol = 1e-6 if _prec(case) == "f" else 1e-14
    assert rel_l2(g, case["grid"].real) < tol
    F = O.compat_bootstrap(case["x"], case.get("y"), ng, nbs, seed, _prec(case))
    assert rel_l2(F, case["F"]) < (1e-6 if _prec(case) == "f" else 1e-13)


def test_hash_known_values(oracle_lib):
    """wang_hash / xorshift32 restated from src/gridding.cu:67-82 on fixed
    inputs (values computed by hand from the published constants)."""
    L = oracle_lib.lib()
    def wang(s):
        s = ((s ^ 61) ^ (s >> 16)) & 0xFFFFFFFF
        s = (s * 9) & 0xFFFFFFFF
        s = s ^ (s >> 4)
        s = (s * 0x27D4EB2D) & 0xFFFFFFFF
        return s ^ (s >> 15)
    def xs(s):
        s ^= (s << 13) & 0xFFFFFFFF
        s ^= s >> 17
        s ^= (s << 5) & 0xFFFFFFFF
        return s & 0xFFFFFFFF
    for s in [0, 1, 12345, 0x7FFFFFFF, 0xFFFFFFFF, 4000000000]:
        assert L.cuna_oracle_wang_hash(s) == wang(s)
        assert L.cuna_oracle_xorshift(s) == xs(s)
        assert L.cuna_oracle_bootstrap_draw(s, 17, 501) == xs(wang((s + 17) & 0xFFFFFFFF)) % 501


def test_cells_bit_exact(oracle_lib):
    """j = (int)((x + 0.5)(ng - 1)) in double, clamped (src/gridding.cu:43-45)."""
    x = np.array([-0.5, 0.5, -0.5000001, 0.5000001, 0.0, 0.25, -0.51, 1e-30], np.float32)
    ng = 256
    want = []
    for v in x:
        j = int(np.trunc((np.float64(v) + 0.5) * (ng - 1)))
        want.append(min(max(j, 0), ng - 1))
    np.testing.assert_array_equal(oracle_lib.compat_cells(x, ng, True), want)


def test_ndft_single_sample(oracle_lib):
    t = np.array([0.3]); y = np.array([1.0]); k = np.arange(-5, 6)
    F = oracle_lib.ndft(t, y, 0.0, 1.0, k)
    np.testing.assert_allclose(F, np.exp(2j * np.pi * k * (0.3 - 0.5)), atol=1e-15)


@pytest.mark.parametrize("n,nf,R,m,tol", [(2000, 1024, 2, 8, 3e-8), (5000, 4096, 4, 12, 1e-12),
                                          (3000, 2048, 2, 10, 1e-9)])
def test_accurate_restatement_vs_ndft(oracle_lib, n, nf, R, m, tol):
    rng = np.random.default_rng(n)
    t = np.sort(rng.uniform(0, 100, n))
    y = rng.normal(0, 1, n)
    F = oracle_lib.accurate_adjoint(t, y, 0.0, 100.0, nf, R, m)
    D = oracle_lib.ndft(t, y, 0.0, 100.0, np.arange(-nf // 2, nf // 2))
    assert rel_l2(F, D) < tol


def test_cpu_pipeline_matches_oracle(oracle_lib):
    """The timed CPU baseline computes the reference's pipeline."""
    case = [c for c in PLAIN if c["name"].startswith("f32_cfg1")][0]
    ng = int(case["ng"])
    p = oracle_lib.CpuPipeline(len(case["x"]), ng)
    F = p.run(case["x"], case["y"])
    assert rel_l2(F, case["F"]) < 1e-5


# ---------------------------------------------------------------------------
# integer steps per sample (the checkers of the GPU's integer outputs)
# ---------------------------------------------------------------------------

def test_bulk_draws_match_scalar_draws(oracle_lib):
    """The bulk draw restatement agrees with the per-draw one pinned above."""
    assert np.array_equal(oracle_lib.bootstrap_draws_all(11, 37, 5).ravel(), oracle_lib.bootstrap_draws(11, 37, 5))
    assert np.array_equal(oracle_lib.bootstrap_draws_all(0xFFFFFFF0, 3, 20).ravel(),
                          oracle_lib.bootstrap_draws(0xFFFFFFF0, 3, 20))


@pytest.mark.parametrize("case", PLAIN, ids=lambda c: c["name"])
def test_taps_match_pinned_cells_and_filter(oracle_lib, case):
    """compat_taps gives the cells of the pinned compat_cells, and its origin
    u reproduces the golden E1/E2 of the reference's own sources:
    eps = ng x - u lands in [R_f - 1, R_f + 1] for every in-range sample."""
    x = case["x"]
    ng = int(case["ng"])
    dt = x.dtype
    j, u, ms, me = oracle_lib.compat_taps(x, ng, dt, clamp=True)
    assert np.array_equal(j, oracle_lib.compat_cells(x, ng, True))
    rf = int(case["rf"])
    inr = np.abs(x.astype(np.float64)) <= 0.5
    eps = ng * x.astype(np.float64)[inr] - u[inr]
    assert np.all((eps >= rf - 1) & (eps <= rf + 1))
    has = ms < me
    assert np.all(j[has].astype(np.int64) + ms[has] >= 0) and np.all(j[has].astype(np.int64) + me[has] <= ng)


def test_tap_range_edges(oracle_lib):
    """Tap ranges at the grid edges and for cells far outside it."""
    ng = 64
    x = np.array([-0.5, 0.5, 0.0, 2.0, -2.0, 1e9, -1e9, np.inf, -np.inf, np.nan], np.float32)
    j, u, ms, me = oracle_lib.compat_taps(x, ng, np.float32, clamp=False)
    assert (j[0], ms[0], me[0]) == (0, 0, 6)                 # taps 0..5 from cell 0
    assert (j[1], ms[1], me[1]) == (63, -5, 1)               # taps -5..0 from the last cell
    assert ms[3] == me[3] == 0 and ms[4] == me[4] == 0       # outside the grid: no taps
    assert np.all(ms[5:9] == 0) and np.all(me[5:9] == 0)     # |j| > 2^30: no taps
    # NaN: the double cell converts to INT_MIN (no taps), the float origin
    # to 0, as sm_103a converts them
    assert j[9] == -2 ** 31 and u[9] == 0 and ms[9] == me[9] == 0


def test_fixed_point_phase_against_rationals(oracle_lib):
    """The fixed-point phase restatement against exact rational arithmetic:
    S = frac((t - t0)/T) 2^64 to within the rounding of A = 2^64/T to 64
    significant bits (relative 2^-63, so a few units times |t/T| + |t0/T|)
    and the two truncations; the cell is floor(S ng / 2^64)."""
    from fractions import Fraction
    rng = np.random.default_rng(4)
    for t0, T, ng in ((0.0, 3650.0, 1 << 22), (2451545.0, 1234.5678, 1 << 19), (17.25, 3.0, 3 << 20)):
        t = np.concatenate([t0 + np.arange(-3, 4) * T, t0 + rng.integers(0, ng, 64) * (T / ng),
                            t0 + rng.uniform(-5 * T, 5 * T, 64), [0.0, -0.0, 5e-324, -5e-324, 1e-300]])
        S, cell, _, _ = oracle_lib.phases(t, t0, T, ng)
        for ti, si, ci in zip(t, S, cell):
            r = (Fraction(float(ti)) - Fraction(t0)) / Fraction(T)
            exact = (r - (r.numerator // r.denominator)) * 2 ** 64
            diff = (int(si) - int(exact)) % 2 ** 64
            diff = min(diff, 2 ** 64 - diff)
            bound = 4 * (abs(float(ti) / T) + abs(t0 / T)) + 4
            assert diff <= bound, (ti, diff, bound)
            assert ci == (int(si) * ng) >> 64
