"""Long-horizon parity of the CUDA step with the reference itself: the
reference's own runs of 60-105 steps (vortex 32^2 for 100 steps and to
t=1, four-quadrant 32^2, Kelvin-Helmholtz 32^2 with moncen slopes, Sedov
8^3 through its negative-density steps and 16^3, Sod to t=0.2, an SD-only
step function), stored in tests/golden/long/ by make_golden.py --long.
Tolerance: bitwise (np.array_equal) for the dt of every step, the trouble
mask after every step (CRC-32 and count), the final masks and the state
after end_sim; the specification's 1e-10 relative bound after 100 steps is
implied."""
import numpy as np
import pytest

from golden_cases import load_long, long_case_names, run_like_reference, state_matches
from gpu_helpers import product_from_golden

pytestmark = pytest.mark.gpu


def _final_checks(s, data, kw, masks=True):
    if masks and kw.get("update") == "FV" and kw.get("FB", False):
        assert np.array_equal(s.dm.troubles, data["troubles"])
        assert np.array_equal(s.dm.theta, data["theta"], equal_nan=True)
        for d in s.dims:
            assert np.array_equal(getattr(s.dm, f"affected_faces_{d}"), data[f"affected_faces_{d}"])
    assert s.time == float(data["time"]), (s.time, float(data["time"]))
    for key in ("U_sp", "W_cv"):
        ok, info = state_matches(getattr(s.dm, key), data, key)
        assert ok, (key, info)


@pytest.mark.parametrize("name", long_case_names())
def test_gpu_long_horizon_step_by_step(name):
    """The launch-by-launch step (compute_dt + perform_update) with the
    reference's loop around it: every dt and every step's trouble mask."""
    data, kw, meta = load_long(name)
    s = product_from_golden(data, kw, meta)
    limited = s.update == "FV" and s.FB

    def set_dt(v):
        s.dm.dt = v

    s.init_sim()
    dts, crcs, counts = run_like_reference(s, meta, limited, lambda: s.dm.dt, set_dt, lambda: s.time,
                                           lambda: s.dm.troubles)
    s.n_step = len(dts)
    assert np.array_equal(np.array(dts), data["dts"]), (len(dts), len(data["dts"]))
    if limited:
        assert np.array_equal(np.array(counts), data["troubles_count"])
        assert np.array_equal(np.array(crcs, dtype=np.uint32), data["troubles_crc32"])
    s.end_sim()
    _final_checks(s, data, kw)
    s.close()


@pytest.mark.parametrize("name", long_case_names())
def test_gpu_long_horizon_graph_driver(name):
    """The same run through perform_iterations / perform_time_evolution
    (captured step replayed, dt clip on the device)."""
    data, kw, meta = load_long(name)
    s = product_from_golden(data, kw, meta)
    run = meta["run"]
    import warnings
    with warnings.catch_warnings():
        warnings.simplefilter("ignore", RuntimeWarning)
        if "steps" in run:
            s.perform_iterations(run["steps"])
        else:
            s.perform_time_evolution(run["t_end"])
    assert s.n_step == len(data["dts"])
    _final_checks(s, data, kw)
    if "l1_density_error_vs_exact" in data:
        from spd_gb300.initial_conditions import isentropic_vortex
        from spd_gb300.polynomials import quadrature_mean
        shift = run["t_end"]
        # the exact solution sampled with the reference's default quadrature
        # (src/polynomials.py:124-148, as the fixture's figure was made), here
        # with this machine's NumPy transcendentals: equal to 1e-9 relative
        exact = s.crop(quadrature_mean(s.mesh_cv, isentropic_vortex(center=(5.0 + shift, 5.0 + shift)), 2, 0,
                                       light=True)[None])[0]
        err = float(np.mean(np.abs(s.dm.W_cv[0] - exact)))
        want = float(data["l1_density_error_vs_exact"])
        assert abs(err - want) <= 1e-9 * want, (err, want)
    s.close()
