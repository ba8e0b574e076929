"""Failure detection without a GPU fault: non-finite states injected on the
host are reported by status codes and warnings while the steps run as the
reference runs them; invalid calls return error statuses and leave the
context usable."""
import warnings

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _sim(**kw):
    from spd_gb300 import SDADER_Simulator
    from spd_gb300.initial_conditions import four_quadrant
    base = dict(p=2, N=(16, 16), init_fct=four_quadrant, update="FV", FB=True, riemann_solver_sd="hllc",
                riemann_solver_fv="hllc", BC=(("gradfree", "gradfree"),) * 2, verbose=False)
    base.update(kw)
    return SDADER_Simulator(**base)


def test_nan_injection_is_reported_not_hidden():
    s = _sim()
    U = s.dm.U_sp
    U[0, 3, 3, 1, 1] = np.nan
    s.dm.U_sp = U
    W = s.dm.W_cv
    W[0, 3, 3, 1, 1] = np.nan
    s.dm.W_cv = W
    with pytest.warns(RuntimeWarning, match="non-finite dt"):
        s.perform_iterations(2)
    assert s.n_step == 2
    assert np.isnan(s.dm.U_sp).any()
    # the raw driver reports the status with the steps it took
    t, done, nonfinite = s._ctx.step(1, 0.0, 0, s.time)
    assert done == 1 and nonfinite
    s.close()


def test_finite_run_raises_no_warning():
    s = _sim()
    with warnings.catch_warnings():
        warnings.simplefilter("error")
        s.perform_iterations(3)
    assert np.isfinite(s.dm.U_sp).all()
    s.close()


def test_invalid_calls_return_errors_and_keep_the_context_usable():
    from spd_gb300._lib import SpdError
    s = _sim()
    ctx = s._ctx
    with pytest.raises(SpdError):
        ctx.upload("U_sp", np.zeros(7))
    with pytest.raises(SpdError):
        ctx.download("U_sp_adj", s._shape_of("U_sp"))  # adjoint not enabled
    with pytest.raises(SpdError):
        ctx.vjp_step(0)
    ctx.adjoint_enable(2)
    with pytest.raises(SpdError):
        ctx.record_step(2, 1e-3)
    with pytest.raises(SpdError):
        ctx.tape_step(0, 1e-3, 1)  # no tapes
    ctx.tape_enable(1)
    with pytest.raises(SpdError):
        ctx.tape_step(0, 1e-3, 3)
    before = s.dm.U_sp
    s.compute_dt()
    s.perform_update()
    assert np.isfinite(s.dm.U_sp).all() and not np.array_equal(before, s.dm.U_sp)
    s.close()
