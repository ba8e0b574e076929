"""The allocation-free CFL entry point (spd_cfl_dt_noalloc).

Some callers cannot call cudaMalloc: hosts whose framework allocator owns
all device memory, and real-time loops that forbid allocation after
start-up.  spd_cfl_dt_noalloc serves them with
a fixed scratch array inside the library; this test checks, through the C
ABI, that it returns the same dt as the context's own compute_dt, bit for
bit (the tolerance of every parity test here), on two calls in a row.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _entry():
    from spd_gb300 import _lib
    fn = _lib.load().spd_cfl_dt_noalloc
    fn.argtypes = [ctypes.c_void_p, ctypes.c_longlong, ctypes.c_int, ctypes.c_double, ctypes.c_double,
                   ctypes.c_double, ctypes.c_double, ctypes.c_void_p, ctypes.c_void_p]
    fn.restype = ctypes.c_int
    return fn


def test_cfl_dt_noalloc_matches_compute_dt_twice():
    import torch
    from spd_gb300 import SDADER_Simulator
    from spd_gb300.initial_conditions import four_quadrant
    s = SDADER_Simulator(p=3, N=(64, 64), init_fct=four_quadrant, update="FV", FB=True, riemann_solver_sd="hllc",
                         riemann_solver_fv="hllc", BC=(("gradfree", "gradfree"),) * 2, verbose=False)
    fn = _entry()
    h = s.h_min / (s.p + 1)
    out = torch.full((1,), -1.0, dtype=torch.float64, device="cuda")
    for call in range(2):
        if call == 1:
            s.perform_update()  # a different state for the second call
        s.compute_dt()
        expected = s.dm.dt
        W = torch.from_numpy(np.ascontiguousarray(s.transpose_to_fv(s.dm.W_cv))).cuda()
        stream = torch.cuda.current_stream().cuda_stream
        rc = fn(W.data_ptr(), W[0].numel(), s.ndim, s.gamma, s.min_c2, s.cfl_coeff, h, out.data_ptr(), stream)
        assert rc == 0
        torch.cuda.synchronize()
        assert out.item() == expected, (call, out.item(), expected)
    s.close()


def test_cfl_dt_noalloc_partial_last_block_and_nan():
    """30x30 cells at p=2: 8,100 subcells, so the last 256-thread block is
    partly empty (its idle threads contribute 0).  Then a NaN planted in one
    subcell on the host must come back as a NaN dt, as from compute_dt."""
    import math
    import torch
    from spd_gb300 import SDADER_Simulator
    from spd_gb300.initial_conditions import four_quadrant
    s = SDADER_Simulator(p=2, N=(30, 30), init_fct=four_quadrant, update="FV", FB=True, riemann_solver_sd="hllc",
                         riemann_solver_fv="hllc", BC=(("gradfree", "gradfree"),) * 2, verbose=False)
    fn = _entry()
    h = s.h_min / (s.p + 1)
    out = torch.full((1,), -1.0, dtype=torch.float64, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    for call in range(2):
        if call == 1:
            s.perform_update()
        s.compute_dt()
        expected = s.dm.dt
        W = torch.from_numpy(np.ascontiguousarray(s.transpose_to_fv(s.dm.W_cv))).cuda()
        assert W[0].numel() % 256 != 0
        rc = fn(W.data_ptr(), W[0].numel(), s.ndim, s.gamma, s.min_c2, s.cfl_coeff, h, out.data_ptr(), stream)
        assert rc == 0
        torch.cuda.synchronize()
        assert out.item() == expected, (call, out.item(), expected)
    # a NaN density or pressure becomes the sound-speed floor (np.where(c2 >
    # min_c2, c2, min_c2) keeps min_c2 for NaN, src/hydro.py:3-25): dt stays
    # finite and equal; a NaN velocity reaches the maximum and dt is NaN
    for var, want_nan in ((0, False), (1, True)):
        W_sd = s.dm.W_cv
        W_sd[var, 17, 3, 1, 2] = np.nan  # one subcell (SD layout)
        s.dm.W_cv = W_sd
        s.compute_dt()
        expected = s.dm.dt
        assert math.isnan(expected) == want_nan
        W = torch.from_numpy(np.ascontiguousarray(s.transpose_to_fv(W_sd))).cuda()
        rc = fn(W.data_ptr(), W[0].numel(), s.ndim, s.gamma, s.min_c2, s.cfl_coeff, h, out.data_ptr(), stream)
        assert rc == 0
        torch.cuda.synchronize()
        got = out.item()
        assert (math.isnan(got) and want_nan) or got == expected, (var, got, expected)
    s.close()


def test_cfl_dt_noalloc_rejects_oversized_input():
    import torch
    fn = _entry()
    W = torch.ones(4, dtype=torch.float64, device="cuda")
    out = torch.zeros(1, dtype=torch.float64, device="cuda")
    rc = fn(W.data_ptr(), 4194304 + 1, 2, 1.4, 1e-10, 0.8, 0.1, out.data_ptr(), None)
    assert rc == 1  # SPD_ERR_ARG, nothing launched
