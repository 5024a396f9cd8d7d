"""Argument checks of the C ABI's plan constructors, run on the CPU: every
case is refused before any device call, with the documented status code and
a message naming the offending value (for batches, the offending series).
No case reaches the GPU, so these run without one."""
import ctypes

import numpy as np
import pytest

INVALID, UNSUPPORTED = 1, 3
F32, F64 = 0, 1


@pytest.fixture(scope="module")
def core(native_built):
    from cunfft_adjoint_gb300 import _lib
    return _lib.core()


def _arr(values, ctype):
    return (ctype * len(values))(*values)


@pytest.mark.parametrize("dtype,nf,R,m,code,needle", [
    (7, 1024, 2, 8, INVALID, b"dtype"),
    (F32, 1023, 2, 8, INVALID, b"even nf"),
    (F32, 0, 2, 8, INVALID, b"even nf"),
    (F32, 1024, 1, 8, INVALID, b"R >= 2"),
    (F32, 1024, 2, 0, INVALID, b"1 <= m <= 16"),
    (F32, 1024, 2, 17, INVALID, b"1 <= m <= 16"),
    (F32, 1000, 2, 8, UNSUPPORTED, b"power of two"),
    (F32, 1024, 3, 8, UNSUPPORTED, b"power of two"),
    (F32, 8, 2, 8, INVALID, b"smaller than 4m"),
    (F64, 1 << 24, 2, 8, UNSUPPORTED, b"too large"),
    (F32, 1 << 26, 2, 8, UNSUPPORTED, b"too large"),
])
def test_plan_create_rejects(core, dtype, nf, R, m, code, needle):
    plan = ctypes.c_void_p(123)
    st = core.cuna2_plan_create(ctypes.byref(plan), dtype, nf, R, m)
    assert st == code
    assert needle in core.cuna2_last_error()
    assert plan.value is None  # the handle is cleared on failure


def test_plan_create_null_handle(core):
    assert core.cuna2_plan_create(None, F32, 1024, 2, 8) == INVALID
    assert b"NULL" in core.cuna2_last_error()


def _create_ex(core, n, nf, R, m, dtype=F32):
    plan = ctypes.c_void_p(123)
    k = len(n)
    st = core.cuna2_batch_plan_create_ex(ctypes.byref(plan), dtype, k, _arr(n, ctypes.c_int64),
                                         _arr(nf, ctypes.c_int64), _arr(R, ctypes.c_int), _arr(m, ctypes.c_int),
                                         None, None)
    return st, plan


@pytest.mark.parametrize("R,m,nf,needle", [
    ([2, 1, 2], [8, 8, 8], [1024, 1024, 1024], b"series 1"),
    ([2, 2, 2], [8, 8, 17], [1024, 1024, 1024], b"series 2"),
    ([2, 2, 2], [0, 8, 8], [1024, 1024, 1024], b"series 0"),
    ([2, 2, 2], [8, 8, 8], [1024, 1023, 1024], b"series 1"),
    ([2, 2, 2], [8, 8, 8], [1024, 1024, 3000], b"series 2"),
    ([2, 2, 8], [8, 8, 8], [1024, 1024, 1 << 24], b"series 2"),
])
def test_batch_create_ex_names_the_bad_series(core, R, m, nf, needle):
    st, plan = _create_ex(core, [100, 200, 300], nf, R, m)
    assert st == INVALID
    assert needle in core.cuna2_last_error()
    assert plan.value is None


def test_batch_create_rejects_null_arrays_and_scalars(core):
    plan = ctypes.c_void_p()
    n = _arr([10, 20], ctypes.c_int64)
    nf = _arr([256, 256], ctypes.c_int64)
    assert core.cuna2_batch_plan_create_ex(ctypes.byref(plan), F32, 2, n, nf, None, None, None, None) == INVALID
    assert core.cuna2_batch_plan_create_ex(ctypes.byref(plan), F32, 0, n, nf, None, None, None, None) == INVALID
    assert core.cuna2_batch_plan_create(ctypes.byref(plan), F32, 2, n, None, 2, 8, None, None) == INVALID
    assert core.cuna2_batch_plan_create(ctypes.byref(plan), F32, 2, n, nf, 1, 8, None, None) == INVALID
    assert core.cuna2_batch_plan_create(ctypes.byref(plan), F32, 2, n, nf, 2, 17, None, None) == INVALID
    assert core.cuna2_batch_plan_create(ctypes.byref(plan), 5, 2, n, nf, 2, 8, None, None) == INVALID
    assert core.cuna2_batch_plan_create(None, F32, 2, n, nf, 2, 8, None, None) == INVALID


@pytest.mark.parametrize("tol", [0.0, -1e-5, 1.0, 2.0, float("nan")])
def test_batch_create_auto_rejects_bad_tolerance(core, tol):
    plan = ctypes.c_void_p(123)
    n = _arr([10, 20], ctypes.c_int64)
    nf = _arr([256, 256], ctypes.c_int64)
    dummy = ctypes.c_void_p(16)  # never dereferenced: the tolerance is refused first
    Rs, ms = _arr([0, 0], ctypes.c_int), _arr([0, 0], ctypes.c_int)
    st = core.cuna2_batch_plan_create_auto(ctypes.byref(plan), F32, 2, n, nf, tol, None, None, dummy, dummy, dummy,
                                           None, Rs, ms)
    assert st == INVALID
    assert plan.value is None
    assert list(Rs) == [0, 0] and list(ms) == [0, 0]


def test_batch_handles_reject_null(core):
    R = np.zeros(2, np.int32)
    assert core.cuna2_batch_get_filter(None, R.ctypes.data, None) == INVALID
    assert core.cuna2_batch_set_schedule(None, 12, 2) == INVALID
    assert b"NULL plan" in core.cuna2_last_error()


@pytest.mark.parametrize("tol", [0.0, 1.0, float("nan")])
def test_plan_create_auto_rejects_bad_tolerance(core, tol):
    plan = ctypes.c_void_p(123)
    dummy = ctypes.c_void_p(16)  # never dereferenced: the tolerance is refused first
    R, m = ctypes.c_int(0), ctypes.c_int(0)
    st = core.cuna2_plan_create_auto(ctypes.byref(plan), F32, 1024, tol, dummy, dummy, dummy, 10, 0.0, 1.0, None,
                                     ctypes.byref(R), ctypes.byref(m))
    assert st == INVALID
    assert plan.value is None
    assert (R.value, m.value) == (0, 0)
