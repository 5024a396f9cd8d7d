"""CPU tests of the drop-in libraries' host-side functions against fixtures of
the reference's own src/utils.cu (tests/golden/host/host_utils.npz, made by
tests/golden/make_golden.py from the reference sources built for the CPU).

scale_x (src/utils.cu:84-93) must give the reference's bits, including its
habit of subtracting the already-rewritten x[0]; nextPowerOfTwo
(src/utils.cu:55-65) must wrap the same way.  Both are pure host code, so
these run without a GPU through the exported C++ names.
"""
import ctypes
import os

import numpy as np
import pytest

from conftest import GOLDEN_DIR

HOST = np.load(os.path.join(GOLDEN_DIR, "host", "host_utils.npz"))


@pytest.fixture(scope="module")
def libs(native_built):
    from cunfft_adjoint_gb300 import _lib
    return {"f": _lib.dropin("f"), "d": _lib.dropin("d")}


def _cases(prec):
    i = 0
    while "scale_x_%s_%d_in" % (prec, i) in HOST:
        yield i, HOST["scale_x_%s_%d_in" % (prec, i)], HOST["scale_x_%s_%d_out" % (prec, i)]
        i += 1


@pytest.mark.parametrize("prec", ["f", "d"])
def test_scale_x_matches_reference(libs, prec):
    fn = getattr(libs[prec], "_Z7scale_xP%si" % prec)
    fn.argtypes = [ctypes.c_void_p, ctypes.c_int]
    n = 0
    for i, x_in, want in _cases(prec):
        x = np.array(x_in, copy=True)
        fn(x.ctypes.data_as(ctypes.c_void_p), len(x))
        # bit-for-bit, NaN included (a one-element array divides by zero)
        assert np.array_equal(x.view(np.uint32 if prec == "f" else np.uint64),
                              want.view(np.uint32 if prec == "f" else np.uint64)), (prec, i, x, want)
        n += 1
    assert n >= 8


def test_scale_x_first_element_quirk(libs):
    """The reference rewrites x[0] to -1/2 first and subtracts that from the
    rest: [3, 4, 5, 7] -> [-1/2, 5/8, 7/8, 11/8]."""
    fn = libs["f"]._Z7scale_xPfi
    fn.argtypes = [ctypes.c_void_p, ctypes.c_int]
    x = np.array([3, 4, 5, 7], np.float32)
    fn(x.ctypes.data_as(ctypes.c_void_p), 4)
    assert x.tolist() == [-0.5, 0.625, 0.875, 1.375]


def test_scale_x_empty_is_a_no_op(libs):
    fn = libs["d"]._Z7scale_xPdi
    fn.argtypes = [ctypes.c_void_p, ctypes.c_int]
    x = np.array([1.0, 2.0])
    fn(x.ctypes.data_as(ctypes.c_void_p), 0)
    assert x.tolist() == [1.0, 2.0]


@pytest.mark.parametrize("prec", ["f", "d"])
def test_next_power_of_two_matches_reference(libs, prec):
    fn = libs[prec]._Z14nextPowerOfTwoj
    fn.argtypes = [ctypes.c_uint]
    fn.restype = ctypes.c_uint
    got = np.array([fn(int(v)) for v in HOST["next_pow2_in"]], np.uint32)
    assert np.array_equal(got, HOST["next_pow2_out"])
