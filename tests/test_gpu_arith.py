"""The kernels' integer-pipe binary64 multiply against the FP64 unit."""
import ctypes

import pytest

pytestmark = pytest.mark.gpu


def test_integer_pipe_multiply_matches_fp64_unit():
    from spd_gb300 import _lib
    lib = _lib.load()
    fn = lib.spd_selftest_fp64
    fn.argtypes = [ctypes.c_longlong, ctypes.c_ulonglong, ctypes.POINTER(ctypes.c_ulonglong)]
    fn.restype = ctypes.c_int
    bad = ctypes.c_ulonglong(123)
    assert fn(400_000_000, 20261203, ctypes.byref(bad)) == 0
    assert bad.value == 0
