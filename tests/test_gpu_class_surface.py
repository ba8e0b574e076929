"""The reference's class surface on the GPU: SD_Simulator built on its own
(src/sd_simulator.py:19-57, stepping with the SD update), the flux-point
array the reference keeps after a step with the FV update (dm.F_ader_fp_<d>,
src/sdader_simulator.py:297-298) and the derivative helpers built on it
(src/sd_simulator.py:199-206).  Bitwise against the oracle."""
import numpy as np
import pytest

from gpu_helpers import compare, oracle_like, step_both

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("N", [(6,), (6, 6), (6, 6, 6)])
def test_sd_simulator_on_its_own(N):
    from spd_gb300 import SD_Simulator
    s = SD_Simulator("hllc", "SD", p=3, N=N, verbose=False)  # riemann_solver_sd, update positionally
    assert s.riemann_solver_sd_name == "hllc" and s.FB is False
    o = oracle_like(s)
    dts = step_both(s, o, 2)
    assert all(a == b for a, b in dts)
    assert not compare(s, o)
    s.close()


@pytest.mark.parametrize("N,p", [((8,), 2), ((6, 5), 3), ((4, 3, 5), 2)])
def test_flux_point_arrays_after_an_fv_step(N, p):
    from spd_gb300 import SDADER_Simulator
    from spd_gb300 import initial_conditions as ics
    init = ics.four_quadrant if len(N) == 2 else ics.sine_wave
    s = SDADER_Simulator(p=p, N=N, init_fct=init, update="FV", FB=True, riemann_solver_sd="hllc",
                         riemann_solver_fv="hllc", verbose=False)
    o = oracle_like(s)
    step_both(s, o, 1)
    want = o.integrate_faces(o.F_ader)
    for d in s.dims:
        idim = s.dims[d]
        got = getattr(s.dm, f"F_ader_fp_{d}")
        assert got.shape == s.array_fp(dims=d, ader=True).shape
        assert np.array_equal(got, want[idim]), d
        deriv = getattr(s, f"compute_sp_from_dfp_{d}")()
        ref = s.compute_sp_from_dfp(want[idim], d, ader=True) / s.h[d]
        assert np.array_equal(deriv, ref)
    s.close()


def test_flux_point_arrays_absent_with_the_sd_update():
    from spd_gb300 import SDADER_Simulator
    s = SDADER_Simulator(p=2, N=(4, 4), update="SD", verbose=False)
    with pytest.raises(AttributeError, match="update='FV'"):
        s.dm.F_ader_fp_x
    s.close()


@pytest.mark.parametrize("p", [1, 3])
@pytest.mark.parametrize("ndim", [1, 2, 3])
@pytest.mark.parametrize("n", [1, 6])
def test_transforms_round_trip_and_direction_symmetry(p, ndim, n):
    """What the reference's test/test_transforms.py checks, on SD_Simulator
    built with the device context (including single-element grids): the
    subcell and flux-point transforms invert each other to 1e-14, and the
    x and y flux-point interpolations agree up to the transposition.  The
    single-element grid then also steps, bitwise as the oracle."""
    from spd_gb300 import SD_Simulator
    s = SD_Simulator(p=p, N=(n,) * ndim, verbose=False)
    W_cv = s.dm.W_cv
    assert np.all(np.abs(s.compute_cv_from_sp(s.compute_sp_from_cv(W_cv)) - W_cv) < 1e-14)
    W_sp = s.dm.W_sp
    assert np.all(np.abs(s.compute_sp_from_fp(s.compute_fp_from_sp(W_sp, "x"), "x") - W_sp) < 1e-14)
    if ndim == 2:
        W_x = s.transpose_to_fv(s.compute_fp_from_sp(W_sp, "x"))
        W_y = np.transpose(s.transpose_to_fv(s.compute_fp_from_sp(W_sp, "y")), (0, 2, 1))
        assert np.all(np.abs(W_x - W_y) < 1e-14)
    o = oracle_like(s)
    dts = step_both(s, o, 2)
    assert all(a == b for a, b in dts)
    assert not compare(s, o)
    s.close()
