"""numpy/ctypes front end of the CPU oracle.  TEST INFRASTRUCTURE.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline legs import
this module, to verify results or as the timed CPU baseline.  The product never
imports it.

* ``build()`` compiles oracle/cuna_oracle.c into oracle/liboracle.so (gcc).
* ``compat_*``: restatement of the reference library's arithmetic
  (src/gaussian_filter.cu, src/gridding.cu, src/cuna_kernel.cu).
* ``accurate_adjoint``: double-precision restatement of accurate mode.
* ``ndft``: FP64 direct adjoint NDFT, the accuracy oracle.
* ``RefCPU``: the reference library's own sources built for the CPU by
  oracle/build_ref.py (present only where the reference tree was available).
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "liboracle.so")
SRC = os.path.join(HERE, "cuna_oracle.c")

_lib = None


def build(force=False):
    if force or not os.path.exists(LIB) or os.path.getmtime(LIB) < os.path.getmtime(SRC):
        subprocess.run(["gcc", "-O2", "-fopenmp", "-fPIC", "-shared", "-ffp-contract=off",
                        "-o", LIB, SRC, "-lm"], check=True)
    return LIB


def lib():
    global _lib
    if _lib is None:
        build()
        _lib = ctypes.CDLL(LIB)
        _declare(_lib)
    return _lib


_P = ctypes.c_void_p
_I = ctypes.c_int
_I64 = ctypes.c_int64
_D = ctypes.c_double
_F = ctypes.c_float
_U = ctypes.c_uint32


def _declare(L):
    L.cuna_oracle_wang_hash.argtypes = [_U]; L.cuna_oracle_wang_hash.restype = _U
    L.cuna_oracle_xorshift.argtypes = [_U]; L.cuna_oracle_xorshift.restype = _U
    L.cuna_oracle_bootstrap_draw.argtypes = [_U, _I, _I]; L.cuna_oracle_bootstrap_draw.restype = _I
    L.cuna_oracle_compat_cell.argtypes = [_D, _I, _I]; L.cuna_oracle_compat_cell.restype = _I
    L.cuna_oracle_compat_filter_f32.argtypes = [_P, _I, _I, _P, _P, _P, _P, _P, _P]
    L.cuna_oracle_compat_filter_f64.argtypes = [_P, _I, _I, _P, _P, _P, _P, _P, _P]
    L.cuna_oracle_compat_grid_f32.argtypes = [_P, _P, _I, _I, _P, _P, _P, _I, _P]
    L.cuna_oracle_compat_grid_f64.argtypes = [_P, _P, _I, _I, _P, _P, _P, _I, _P]
    L.cuna_oracle_compat_grid_bootstrap_f32.argtypes = [_P, _P, _I, _I, _I, _P, _P, _P, _I, _U, _P]
    L.cuna_oracle_compat_grid_bootstrap_f64.argtypes = [_P, _P, _I, _I, _I, _P, _P, _P, _I, _U, _P]
    L.cuna_oracle_compat_norm_f32.argtypes = [_I, _F, _F, _P]
    L.cuna_oracle_compat_norm_f64.argtypes = [_I, _D, _D, _P]
    L.cuna_oracle_fft.argtypes = [_P, _I64, _I]
    L.cuna_oracle_accurate_tau.argtypes = [_I, _D]; L.cuna_oracle_accurate_tau.restype = _D
    L.cuna_oracle_accurate_adjoint.argtypes = [_P, _P, _I64, _D, _D, _I64, _I, _I, _P]
    L.cuna_oracle_ndft.argtypes = [_P, _P, _P, _I64, _D, _D, _P, _I64, _P]
    L.cuna_oracle_ndft_grad.argtypes = [_P, _P, _I64, _D, _D, _P, _P, _I64, _P, _P]
    L.cuna_oracle_num_threads.restype = _I
    L.cuna_oracle_cpu_pipeline_f32.argtypes = [_P, _P, _I, _I, _P, _P, _P, _P, _P]
    L.cuna_oracle_cpu_twiddles_f32.argtypes = [_I64, _P]


def _p(a):
    return None if a is None else a.ctypes.data_as(ctypes.c_void_p)


def _dt(prec):
    return np.float32 if prec in ("f", "f32", np.float32) else np.float64


# --------------------------------------------------------------------------
# compat restatement
# --------------------------------------------------------------------------

def compat_filter(x, ng, prec):
    """(b, normfac, rf, E1, E2, E3) as generate_filter_properties computes them."""
    dt = _dt(prec)
    x = np.ascontiguousarray(x, dtype=dt)
    n = len(x)
    rf = 6 if dt == np.float32 else 12
    E1 = np.empty(n, dt); E2 = np.empty(n, dt); E3 = np.empty(rf, dt)
    b = np.zeros(1, dt); nf = np.zeros(1, dt); r = np.zeros(1, np.int32)
    fn = lib().cuna_oracle_compat_filter_f32 if dt == np.float32 else lib().cuna_oracle_compat_filter_f64
    fn(_p(x), n, ng, _p(b), _p(nf), _p(r), _p(E1), _p(E2), _p(E3))
    return b[0], nf[0], int(r[0]), E1, E2, E3


def compat_cells(x, ng, clamp=True):
    L = lib()
    return np.array([L.cuna_oracle_compat_cell(float(v), ng, 1 if clamp else 0) for v in x], np.int64)


def compat_grid(x, y, ng, prec):
    """Real part of the grid after fast_gridding (double accumulation)."""
    dt = _dt(prec)
    x = np.ascontiguousarray(x, dtype=dt)
    y = None if y is None else np.ascontiguousarray(y, dtype=dt)
    b, nf, rf, E1, E2, E3 = compat_filter(x, ng, dt)
    g = np.zeros(ng, np.float64)
    fn = lib().cuna_oracle_compat_grid_f32 if dt == np.float32 else lib().cuna_oracle_compat_grid_f64
    fn(_p(x), _p(y), len(x), ng, _p(E1), _p(E2), _p(E3), rf, _p(g))
    return g


def compat_grid_bootstrap(x, y, ng, nbs, seed, prec):
    dt = _dt(prec)
    x = np.ascontiguousarray(x, dtype=dt)
    y = None if y is None else np.ascontiguousarray(y, dtype=dt)
    b, nf, rf, E1, E2, E3 = compat_filter(x, ng, dt)
    g = np.zeros(nbs * ng, np.float64)
    fn = (lib().cuna_oracle_compat_grid_bootstrap_f32 if dt == np.float32
          else lib().cuna_oracle_compat_grid_bootstrap_f64)
    fn(_p(x), _p(y), len(x), ng, nbs, _p(E1), _p(E2), _p(E3), rf, seed & 0xFFFFFFFF, _p(g))
    return g.reshape(nbs, ng)


def compat_norm(ng, b, normfac, prec):
    dt = _dt(prec)
    fac = np.empty(ng, np.float64)
    if dt == np.float32:
        lib().cuna_oracle_compat_norm_f32(ng, float(b), float(normfac), _p(fac))
    else:
        lib().cuna_oracle_compat_norm_f64(ng, float(b), float(normfac), _p(fac))
    return fac


def fft_inverse(a):
    """Unnormalised CUFFT_INVERSE-convention DFT (e^{+2 pi i n k / N}) in double."""
    a = np.ascontiguousarray(a, dtype=np.complex128).copy()
    buf = a.view(np.float64)
    lib().cuna_oracle_fft(_p(buf), len(a), 1)
    return a


def compat_adjoint(x, y, ng, prec, f_hat0=None):
    """cunfft_adjoint_raw: gridding into f_hat0 (default zeros), inverse FFT,
    deconvolution.  Returns complex128 of length ng."""
    g = compat_grid(x, y, ng, prec)
    b, nf, rf, *_ = compat_filter(x, ng, prec)
    a = g.astype(np.complex128)
    if f_hat0 is not None:
        a = a + np.asarray(f_hat0, np.complex128)
    a = fft_inverse(a)
    return a * compat_norm(ng, b, nf, prec)


def compat_bootstrap(x, y, ng, nbs, seed, prec, f_hat0=None):
    g = compat_grid_bootstrap(x, y, ng, nbs, seed, prec).astype(np.complex128)
    if f_hat0 is not None:
        g = g + np.asarray(f_hat0, np.complex128).reshape(nbs, ng)
    b, nf, rf, *_ = compat_filter(x, ng, prec)
    fac = compat_norm(ng, b, nf, prec)
    return np.stack([fft_inverse(row) * fac for row in g])


def bootstrap_draws(seed, n, nbs):
    L = lib()
    return np.array([L.cuna_oracle_bootstrap_draw(seed & 0xFFFFFFFF, i, n) for i in range(n * nbs)],
                    np.int64)


# --------------------------------------------------------------------------
# accurate mode + NDFT
# --------------------------------------------------------------------------

def accurate_tau(m, R):
    return lib().cuna_oracle_accurate_tau(m, float(R))


def accurate_adjoint(t, y, t0, T, nf, R, m):
    t = np.ascontiguousarray(t, np.float64)
    y = np.ascontiguousarray(y, np.float64)
    F = np.empty(nf, np.complex128)
    lib().cuna_oracle_accurate_adjoint(_p(t), _p(y), len(t), float(t0), float(T), nf, R, m,
                                       _p(F.view(np.float64)))
    return F


def ndft(t, y, t0, T, k):
    """F[q] = sum_j y_j exp(+2 pi i k_q x_j), x_j = (t_j - t0)/T - 1/2 (FP64)."""
    t = np.ascontiguousarray(t, np.float64)
    y = np.asarray(y)
    yr = np.ascontiguousarray(y.real, np.float64)
    yi = np.ascontiguousarray(y.imag, np.float64) if np.iscomplexobj(y) else None
    k = np.ascontiguousarray(k, np.int64)
    F = np.empty(len(k), np.complex128)
    lib().cuna_oracle_ndft(_p(t), _p(yr), _p(yi), len(t), float(t0), float(T), _p(k), len(k),
                           _p(F.view(np.float64)))
    return F


def ndft_grad(t, y, t0, T, k, g):
    """FP64 gradient (dL/dy, dL/dt) of a real loss through the direct adjoint
    NDFT, given g_q = dL/dRe F_q + i dL/dIm F_q on frequencies k_q."""
    t = np.ascontiguousarray(t, np.float64)
    y = np.ascontiguousarray(y, np.float64)
    k = np.ascontiguousarray(k, np.int64)
    g = np.ascontiguousarray(g, np.complex128)
    gy = np.empty(len(t)); gt = np.empty(len(t))
    lib().cuna_oracle_ndft_grad(_p(t), _p(y), len(t), float(t0), float(T), _p(k), _p(g.view(np.float64)),
                                len(k), _p(gy), _p(gt))
    return gy, gt


def num_threads():
    return lib().cuna_oracle_num_threads()


class CpuPipeline:
    """The reference pipeline (compat math, float) as a multi-threaded CPU
    program; used as the timed CPU baseline."""

    def __init__(self, n, ng):
        assert ng & (ng - 1) == 0, "CPU pipeline FFT needs a power-of-two grid"
        self.n, self.ng = n, ng
        nt = num_threads()
        self.f_hat = np.zeros(2 * ng, np.float32)
        self.E1 = np.empty(n, np.float32)
        self.E2 = np.empty(n, np.float32)
        self.work = np.empty(nt * ng, np.float32)
        self.tw = np.empty(ng, np.float32)
        lib().cuna_oracle_cpu_twiddles_f32(ng, _p(self.tw))

    def run(self, x, y):
        x = np.ascontiguousarray(x, np.float32)
        y = np.ascontiguousarray(y, np.float32)
        lib().cuna_oracle_cpu_pipeline_f32(_p(x), _p(y), self.n, self.ng, _p(self.f_hat),
                                           _p(self.E1), _p(self.E2), _p(self.work), _p(self.tw))
        return self.f_hat.view(np.complex64)


# --------------------------------------------------------------------------
# the reference's own sources, built for the CPU (oracle/build_ref.py)
# --------------------------------------------------------------------------

class RefCPU:
    """ctypes view of oracle/_ref/libcuna_refcpu_{f,d}.so."""

    def __init__(self, prec):
        self.dt = _dt(prec)
        tag = "f" if self.dt == np.float32 else "d"
        path = os.path.join(HERE, "_ref", "libcuna_refcpu_%s.so" % tag)
        if not os.path.exists(path):
            raise FileNotFoundError(path)
        self.L = ctypes.CDLL(path)
        self.ct = np.complex64 if self.dt == np.float32 else np.complex128
        L = self.L
        L.refcpu_filter_properties.argtypes = [_P, _I, _I, _P, _P, _P, _P, _P, _P]
        L.refcpu_fast_gridding.argtypes = [_P, _P, _P, _I, _I]
        L.refcpu_fast_gridding_bootstrap.argtypes = [_P, _P, _P, _I, _I, _I, _U]
        L.refcpu_adjoint_raw.argtypes = [_P, _P, _P, _I, _I]
        L.refcpu_adjoint_raw_async.argtypes = [_P, _P, _P, _I, _I]
        L.refcpu_adjoint_bootstrap.argtypes = [_P, _P, _P, _I, _I, _I, _U]
        L.refcpu_plan_adjoint.argtypes = [_P, _P, _I, _I, _U, _P, _P]
        tag_f = "f" if self.dt == np.float32 else "d"
        self._scale_x = getattr(L, "_Z7scale_xP%si" % tag_f)
        self._scale_x.argtypes = [_P, _I]
        self._next_pow2 = L._Z14nextPowerOfTwoj
        self._next_pow2.argtypes = [_U]
        self._next_pow2.restype = _U

    @staticmethod
    def available(prec="f"):
        tag = "f" if _dt(prec) == np.float32 else "d"
        return os.path.exists(os.path.join(HERE, "_ref", "libcuna_refcpu_%s.so" % tag))

    def _in(self, a):
        return None if a is None else np.ascontiguousarray(a, dtype=self.dt)

    def filter_properties(self, x, ng):
        x = self._in(x); n = len(x)
        rf = 6 if self.dt == np.float32 else 12
        E1 = np.empty(n, self.dt); E2 = np.empty(n, self.dt); E3 = np.empty(rf, self.dt)
        b = np.zeros(1, self.dt); nf = np.zeros(1, self.dt); r = np.zeros(1, np.int32)
        self.L.refcpu_filter_properties(_p(x), n, ng, _p(b), _p(nf), _p(r), _p(E1), _p(E2), _p(E3))
        return b[0], nf[0], int(r[0]), E1, E2, E3

    def fast_gridding(self, x, y, ng, f_hat0=None):
        x = self._in(x); y = self._in(y)
        f = np.zeros(ng, self.ct) if f_hat0 is None else np.array(f_hat0, self.ct)
        self.L.refcpu_fast_gridding(_p(x), _p(y), _p(f), len(x), ng)
        return f

    def fast_gridding_bootstrap(self, x, y, ng, nbs, seed):
        x = self._in(x); y = self._in(y)
        f = np.zeros(nbs * ng, self.ct)
        self.L.refcpu_fast_gridding_bootstrap(_p(x), _p(y), _p(f), len(x), ng, nbs, seed & 0xFFFFFFFF)
        return f.reshape(nbs, ng)

    def adjoint_raw(self, x, y, ng, f_hat0=None, async_=False):
        x = self._in(x); y = self._in(y)
        f = np.zeros(ng, self.ct) if f_hat0 is None else np.array(f_hat0, self.ct)
        fn = self.L.refcpu_adjoint_raw_async if async_ else self.L.refcpu_adjoint_raw
        fn(_p(x), _p(y), _p(f), len(x), ng)
        return f

    def scale_x(self, x):
        """scale_x (src/utils.cu:84-93) applied in place to a copy of x."""
        x = np.array(x, self.dt)
        self._scale_x(_p(x), len(x))
        return x

    def next_power_of_two(self, v):
        """nextPowerOfTwo (src/utils.cu:55-65)."""
        return int(self._next_pow2(v & 0xFFFFFFFF))

    def plan_adjoint(self, x, y, ng, flags):
        """init_plan + cunfft_adjoint_from_plan + copyResultsToCPU: (f_hat,
        f_hat_win or None)."""
        x = self._in(x); y = self._in(y)
        f = np.zeros(ng, self.ct)
        w = np.zeros(ng, self.ct)
        self.L.refcpu_plan_adjoint(_p(x), _p(y), len(x), ng, flags, _p(f), _p(w))
        return f, (w if flags & 0x04 else None)

    def adjoint_bootstrap(self, x, y, ng, nbs, seed):
        x = self._in(x); y = self._in(y)
        f = np.zeros(nbs * ng, self.ct)
        self.L.refcpu_adjoint_bootstrap(_p(x), _p(y), _p(f), len(x), ng, nbs, seed & 0xFFFFFFFF)
        return f.reshape(nbs, ng)


# --------------------------------------------------------------------------
# integer steps per sample (bit-exact checkers)
# --------------------------------------------------------------------------

def _declare_int(L):
    if getattr(L, "_int_declared", False):
        return
    L.cuna_oracle_compat_taps_f32.argtypes = [_P, _I, _I, _I, _P, _P, _P, _P]
    L.cuna_oracle_compat_taps_f64.argtypes = [_P, _I, _I, _I, _P, _P, _P, _P]
    L.cuna_oracle_bootstrap_draws.argtypes = [_U, _I, _I, _P]
    L.cuna_oracle_phase_setup.argtypes = [_D, _D, _P, _P, _P]
    L.cuna_oracle_phases.argtypes = [_P, _I64, _D, _D, _I64, _P, _P, _P, _P]
    L._int_declared = True


def compat_taps(x, ng, prec, clamp=True):
    """(j, u, ms, me) per sample: the cell of src/gridding.cu:43-45 (clamped
    when `clamp`), the filter origin of src/gaussian_filter.cu:213 and the tap
    range of src/gridding.cu:53-58 ((0, 0) when empty)."""
    L = lib(); _declare_int(L)
    dt = _dt(prec)
    x = np.ascontiguousarray(x, dtype=dt)
    n = len(x)
    out = [np.empty(n, np.int32) for _ in range(4)]
    fn = L.cuna_oracle_compat_taps_f32 if dt == np.float32 else L.cuna_oracle_compat_taps_f64
    fn(_p(x), n, ng, 1 if clamp else 0, *[_p(o) for o in out])
    return tuple(out)


def compat_tiles(j, ms, me, log_tile=12):
    """Tiles a compat sample's taps touch: (first, last) tile of [j+ms, j+me-1]
    with 2^log_tile-cell tiles; rows with an empty range give (-1, -1)."""
    j = np.asarray(j, np.int64); ms = np.asarray(ms, np.int64); me = np.asarray(me, np.int64)
    has = ms < me
    t0 = np.where(has, (j + ms) >> log_tile, -1)
    t1 = np.where(has, (j + me - 1) >> log_tile, -1)
    return t0, t1


def bootstrap_draws_all(seed, n, nbs):
    """d[b, i] for resample b < nbs and draw i < n (src/gridding.cu:101)."""
    L = lib(); _declare_int(L)
    d = np.empty(n * nbs, np.int32)
    L.cuna_oracle_bootstrap_draws(seed & 0xFFFFFFFF, n, nbs, _p(d))
    return d.reshape(nbs, n)


def phase_setup(t0, T):
    L = lib(); _declare_int(L)
    mA = np.zeros(1, np.uint64); eA = np.zeros(1, np.int32); B = np.zeros(1, np.uint64)
    L.cuna_oracle_phase_setup(float(t0), float(T), _p(mA), _p(eA), _p(B))
    return int(mA[0]), int(eA[0]), int(B[0])


def phases(t, t0, T, ng):
    """Accurate mode's grid-index reduction per sample: (S, cell, frac24,
    frac53) with S = frac((t - t0)/T) 2^64 in 64-bit fixed point, cell =
    floor(S ng / 2^64), and the fractional cell's top 24 / 53 bits."""
    L = lib(); _declare_int(L)
    t = np.ascontiguousarray(t, np.float64)
    n = len(t)
    S = np.empty(n, np.uint64); cell = np.empty(n, np.int32)
    f24 = np.empty(n, np.uint32); f53 = np.empty(n, np.uint64)
    L.cuna_oracle_phases(_p(t), n, float(t0), float(T), int(ng), _p(S), _p(cell), _p(f24), _p(f53))
    return S, cell, f24, f53


def accurate_tiles(cell, ng, m, log_tile):
    """(first, last) tile of accurate mode's periodic tap window
    [cell - m + 1, cell + m] (mod ng) with 2^log_tile-cell tiles."""
    cell = np.asarray(cell, np.int64)
    lo = cell - m + 1
    hi = cell + m
    lo = np.where(lo < 0, lo + ng, lo)
    hi = np.where(hi >= ng, hi - ng, hi)
    return lo >> log_tile, hi >> log_tile
