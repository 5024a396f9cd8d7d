"""CPU checks of the float-float exp2 used by float64 plans (common.cuh):

* every entry of the 2^(j/64) table is the value's float-float split (hi the
  nearest float, lo the nearest float to the remainder), to 2^-48 relative;
* the algorithm, replayed step by step in float32 arithmetic (fused
  multiply-adds formed in float64, exact for the float products involved),
  stays within 7e-15 relative of 2^x over |x| < 100, against 120-bit
  arithmetic.

The table is read from the header itself, so the test follows the source.
"""
import os
import re

import numpy as np
import pytest

from conftest import ROOT

mpmath = pytest.importorskip("mpmath")

f32 = np.float32
HEADER = os.path.join(ROOT, "cunfft_adjoint_gb300", "csrc", "common.cuh")


def _table():
    src = open(HEADER).read()
    body = src[src.index("kDfExp2Tab[64] = {"):]
    body = body[:body.index("};")]
    lit = r"(-?0x[0-9a-f.]+p[+-]\d+f|-?0\.0f)"
    pairs = re.findall(r"\{" + lit + r", " + lit + r"\}", body)
    conv = lambda s: f32(float.fromhex(s[:-1])) if "0x" in s else f32(float(s[:-1]))
    return [(conv(a), conv(b)) for a, b in pairs]


def _fma(a, b, c):
    return f32(np.float64(a) * np.float64(b) + np.float64(c))


def _fts(a, b):
    s = f32(a + b)
    return s, f32(b - f32(s - a))


def _add(a, b):
    s = f32(a[0] + b[0])
    v = f32(s - a[0])
    e = f32(f32(a[0] - f32(s - v)) + f32(b[0] - v))
    e = f32(e + f32(a[1] + b[1]))
    return _fts(s, e)


def _mul(a, b):
    p = f32(a[0] * b[0])
    e = _fma(a[0], b[0], -p)
    e = _fma(a[0], b[1], e)
    e = _fma(a[1], b[0], e)
    return _fts(p, e)


def _split(d):
    hi = f32(d)
    return hi, f32(d - float(hi))


def _df_exp2(x, tab):
    kf = f32(np.rint(f32(x[0] * f32(64))))
    k = int(kf)
    r = _add(x, (f32(-f32(kf * f32(0.015625))), f32(0)))
    z = _mul(r, _split(0.69314718055994530942))
    c6 = _mul(z, _split(1.0 / 6.0))
    u2 = f32(f32(z[0] * z[0]) * _fma(z[0], f32(1.0 / 120.0), f32(1.0 / 24.0)))
    sh, sl = _fts(f32(0.5), c6[0])
    s = _fts(sh, f32(sl + f32(c6[1] + u2)))
    em1 = _add(z, _mul(_mul(z, z), s))
    t = tab[k & 63]
    v = _add(t, _mul(t, em1))
    sc = f32(2.0 ** (k >> 6))
    return f32(v[0] * sc), f32(v[1] * sc)


def test_exp2_table_entries():
    mpmath.mp.prec = 120
    tab = _table()
    assert len(tab) == 64
    for j, (hi, lo) in enumerate(tab):
        v = mpmath.power(2, mpmath.mpf(j) / 64)
        assert hi == f32(float(v)), j
        assert lo == f32(float(v - mpmath.mpf(float(hi)))), j
        err = abs(mpmath.mpf(float(hi)) + mpmath.mpf(float(lo)) - v) / v
        assert err < 2.0 ** -48, (j, float(err))


def test_exp2_algorithm_error_bound():
    mpmath.mp.prec = 120
    tab = _table()
    rng = np.random.default_rng(1)
    xs = np.concatenate([rng.uniform(-10, 10, 1500), rng.uniform(-99, 99, 500), rng.uniform(-0.02, 0.02, 300),
                         [0.0, 1 / 128, -1 / 128, 1 / 64, 0.5, -0.5, 99.3, -99.7]])
    worst = 0.0
    for xv in xs:
        hi = f32(xv)
        x = (hi, f32(f32(xv - float(hi)) * f32(0.3)))
        got = _df_exp2(x, tab)
        want = mpmath.power(2, mpmath.mpf(float(x[0])) + mpmath.mpf(float(x[1])))
        err = abs(mpmath.mpf(float(got[0])) + mpmath.mpf(float(got[1])) - want) / want
        worst = max(worst, float(err))
    assert worst < 7e-15, worst
