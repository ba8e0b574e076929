"""perform_iterations and perform_time_evolution replay one captured step
(CUDA graphs: CFL dt with the t_end clip; update with device-side time
accumulation); the result is the launch-by-launch loop's, bit for bit, also
when graph replays and single steps are mixed and when the number of FV
substeps is odd (buffer roles alternate)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _make(p):
    from spd_gb300 import SDADER_Simulator
    from spd_gb300.initial_conditions import four_quadrant
    return SDADER_Simulator(p=p, N=(24, 24), init_fct=four_quadrant, update="FV", FB=True,
                            riemann_solver_sd="hllc", riemann_solver_fv="hllc",
                            BC=(("gradfree", "gradfree"),) * 2, verbose=False)


def _loop(s, n):
    for _ in range(n):
        s.compute_dt()
        s.perform_update()


@pytest.mark.parametrize("p", [2, 3])
def test_graph_steps_equal_launch_by_launch(p):
    a, b = _make(p), _make(p)
    # perform_iterations ends with end_sim (U_cv, W_cv from U_sp), as in the
    # reference; the launch-by-launch run does the same at the same points
    _loop(a, 3)
    a._ctx.end_sim()
    _loop(a, 4)
    a._ctx.end_sim()
    b.perform_iterations(3)   # graph
    _loop(b, 1)               # single step in between
    b.perform_iterations(3)   # graph again
    assert b.n_step == a.n_step == 7
    assert b.time == a.time
    for key in ("U_sp", "U_cv", "W_cv", "troubles", "theta"):
        assert np.array_equal(getattr(a.dm, key), getattr(b.dm, key), equal_nan=True), key
    a.close()
    b.close()


def test_graph_counts_its_kernel_launches():
    s = _make(3)
    s.perform_iterations(1)
    n0 = s._ctx.launch_count()
    s.perform_iterations(4)             # 4 graph steps + end_sim (2 kernels)
    per_step = (s._ctx.launch_count() - n0 - 2) / 4
    s._ctx.profile(True)                # profiling steps launch by launch
    n1 = s._ctx.launch_count()
    s.perform_iterations(1)
    s._ctx.profile(False)
    s._ctx.profile_report()
    single = s._ctx.launch_count() - n1 - 2
    assert per_step == single + 2       # + the device dt clip and time add
    s.close()


@pytest.mark.parametrize("p", [2, 3])
def test_time_evolution_graph_equals_host_loop(p):
    """perform_time_evolution replays the dt graph (with the t_end clip on
    the device) and the update graph; profiling forces the host loop."""
    a, b = _make(p), _make(p)
    a._ctx.profile(True)
    a.perform_time_evolution(0.02)
    a._ctx.profile(False)
    a._ctx.profile_report()
    b.perform_time_evolution(0.02)
    assert a.n_step == b.n_step > 1
    assert a.time == b.time == 0.02
    for key in ("U_sp", "U_cv", "W_cv", "troubles", "theta"):
        assert np.array_equal(getattr(a.dm, key), getattr(b.dm, key), equal_nan=True), key
    a.close()
    b.close()
