"""Parity of the CUDA step with the reference (golden fixtures) and with
the oracle restatement (same inputs, run here).  Floating-point tolerance:
the kernels reproduce the reference's operation order, so every comparison
is bitwise (np.array_equal); the 1e-12 / 1e-10 relative bounds of the
specification are implied."""
import numpy as np
import pytest

from golden_cases import DIMS, case_names, load
from gpu_helpers import compare, oracle_like, product_from_golden, step_both

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name", case_names())
def test_gpu_matches_reference_golden(name):
    data, kw, meta = load(name)
    s = product_from_golden(data, kw, meta)
    dts = []
    for _ in range(meta["steps"]):
        s.compute_dt()
        dts.append(s.dm.dt)
        s.perform_update()
    assert np.array_equal(np.array(dts), data["dts"]), (dts, data["dts"])
    assert s.time == float(data["time"])
    for key in ("U_sp", "U_cv", "W_cv"):
        got = getattr(s.dm, key)
        assert np.array_equal(got, data[key], equal_nan=True), (key, np.nanmax(np.abs(got - data[key])))
    if "troubles" in data:
        assert np.array_equal(s.dm.troubles, data["troubles"])
        assert np.array_equal(s.dm.theta, data["theta"])
        for d in s.dims:
            assert np.array_equal(getattr(s.dm, f"affected_faces_{d}"), data[f"affected_faces_{d}"])
    s.close()


def _run_vs_oracle(nsteps, **kw):
    from spd_gb300 import SDADER_Simulator
    s = SDADER_Simulator(verbose=False, **kw)
    o = oracle_like(s)
    dts = step_both(s, o, nsteps)
    assert all(a == b for a, b in dts), dts[:3]
    bad = compare(s, o)
    troubles = float(s.dm.troubles.sum()) if (s.update == "FV" and s.FB) else 0.0
    s.close()
    return bad, troubles


def test_vortex_32_p3_100_steps_bitwise():
    """Isentropic vortex, 32x32 cells, p=3, FV update with limiting, LLF,
    100 steps (the parity case of the vortex benchmark)."""
    from spd_gb300.initial_conditions import isentropic_vortex
    bad, _ = _run_vs_oracle(100, p=3, N=(32, 32), xlim=(0, 10), ylim=(0, 10), init_fct=isentropic_vortex(),
                            update="FV", FB=True, riemann_solver_sd="llf", riemann_solver_fv="llf",
                            BC=(("periodic", "periodic"),) * 2)
    assert not bad, bad


def test_quadrant_64_p3_100_steps_bitwise():
    """Four-quadrant Riemann problem at 64x64 cells (the 512x512 benchmark
    reduced), transmissive boundaries, HLLC, limiting, 100 steps: state,
    dt and trouble masks bit-identical to the oracle."""
    from spd_gb300.initial_conditions import four_quadrant
    bad, troubles = _run_vs_oracle(100, p=3, N=(64, 64), init_fct=four_quadrant, update="FV", FB=True,
                                   riemann_solver_sd="hllc", riemann_solver_fv="hllc",
                                   BC=(("gradfree", "gradfree"),) * 2)
    assert troubles > 0
    assert not bad, bad


def test_sedov_16_p2_100_steps_bitwise():
    """3D Sedov blast at 16^3 cells (the 128^3 benchmark reduced), p=2,
    reflective walls, HLLC, limiting, 100 steps: state, dt and trouble
    masks bit-identical to the oracle."""
    from spd_gb300.initial_conditions import sedov
    bad, troubles = _run_vs_oracle(100, p=2, N=(16, 16, 16), init_fct=sedov(16), update="FV", FB=True,
                                   riemann_solver_sd="hllc", riemann_solver_fv="hllc",
                                   BC=(("reflective", "reflective"),) * 3)
    assert troubles > 0
    assert not bad, bad


@pytest.mark.parametrize("p", [1, 3])
@pytest.mark.parametrize("N", [(6,), (6, 6), (6, 6, 6)])
@pytest.mark.parametrize("update", ["SD", "FV"])
@pytest.mark.parametrize("FB", [True, False])
def test_update_matrix_vs_oracle(p, N, update, FB):
    """Mirrors the reference's test/test_update.py:10-18 (every dimension,
    degree, update and limiting flag), with a bitwise check."""
    bad, _ = _run_vs_oracle(2, p=p, N=N, update=update, FB=FB)
    assert not bad, bad


@pytest.mark.parametrize("p", [1, 3])
@pytest.mark.parametrize("N", [(6,), (6, 6)])
@pytest.mark.parametrize("mode", ["SD", "FV", "FB_godunov", "FB"])
def test_preserve_velocity_and_pressure(p, N, mode):
    """Mirrors the reference's test/test_preserve.py:10-38: an advected
    density wave keeps velocity and pressure constant.  The threshold is the
    reference's 1e-14 (mean absolute); in 2D with p=3 the reference's own
    NumPy run measures 1.5-1.6e-14 (the same bits as this GPU run), so the
    test asserts equality with the oracle there and 2e-14."""
    from spd_gb300 import SDADER_Simulator
    kw = dict(p=p, N=N, verbose=False)
    if mode == "FV":
        kw["update"] = "FV"
    elif mode == "FB_godunov":
        kw.update(update="FV", FB=True, godunov=True)
    elif mode == "FB":
        kw.update(update="FV", FB=True)
    s = SDADER_Simulator(**kw)
    o = oracle_like(s)
    s.perform_time_evolution(1)
    o.perform_time_evolution(1)
    W = s.dm.W_cv
    assert np.array_equal(W, o.W_cv)
    assert np.mean(np.abs(W[0] - s.W_init_cv[0])) > 1e-14
    tol = 2e-14 if (len(N) == 2 and p == 3) else 1e-14
    assert np.mean(np.abs(W[1:] - s.W_init_cv[1:])) < tol
    s.close()


@pytest.mark.parametrize("p", [1, 3])
@pytest.mark.parametrize("N", [(6,), (6, 6), (6, 6, 6)])
def test_create(p, N):
    """Mirrors the reference's test/test_create.py:12-16."""
    from spd_gb300 import SDADER_Simulator
    s = SDADER_Simulator(p=p, N=N, verbose=False)
    assert s.dm.U_sp.shape == (len(N) + 2,) + N + (p + 1,) * len(N)
    s.close()


def test_vortex_t1_error_against_exact():
    """Vortex benchmark run to t=1: L1 error of the subcell-averaged density
    against the exact (translated) solution, and the same bits as the oracle."""
    from spd_gb300 import SDADER_Simulator
    from spd_gb300.initial_conditions import isentropic_vortex
    from spd_gb300.polynomials import quadrature_mean
    kw = dict(p=3, N=(32, 32), xlim=(0, 10), ylim=(0, 10), update="FV", FB=True, riemann_solver_sd="llf",
              riemann_solver_fv="llf", BC=(("periodic", "periodic"),) * 2, verbose=False)
    s = SDADER_Simulator(init_fct=isentropic_vortex(), **kw)
    o = oracle_like(s)
    s.perform_time_evolution(1.0)
    o.perform_time_evolution(1.0)
    assert s.n_step == 87
    assert np.array_equal(s.dm.U_sp, o.U_sp)
    exact = s.crop(quadrature_mean(s.mesh_cv, isentropic_vortex(center=(6.0, 6.0)), 2, 0, light=False)[None])[0]
    err = float(np.mean(np.abs(s.dm.W_cv[0] - exact)))
    assert 1.0e-6 < err < 2.0e-6, err  # the reference's NumPy run gives 1.556e-6
    assert float(s.dm.troubles.sum()) == 0.0
    s.close()


@pytest.mark.slow
def test_quadrant_512_one_step_full_size_bitwise():
    """The 512x512 four-quadrant benchmark at full size: one step bitwise
    against the oracle (the oracle needs ~10 GB and a minute or two)."""
    from spd_gb300.initial_conditions import four_quadrant
    bad, troubles = _run_vs_oracle(1, p=3, N=(512, 512), init_fct=four_quadrant, update="FV", FB=True,
                                   riemann_solver_sd="hllc", riemann_solver_fv="hllc",
                                   BC=(("gradfree", "gradfree"),) * 2)
    assert troubles > 0
    assert not bad, bad


OPTION_CASES = {
    "p4_fvfb_hllc_gradfree": dict(p=4, N=(8, 8), init="four_quadrant", update="FV", FB=True,
                                  riemann_solver_sd="hllc", riemann_solver_fv="hllc",
                                  BC=(("gradfree", "gradfree"),) * 2),
    "p2_m1_fvfb_llf_periodic": dict(p=2, m=1, N=(8, 8), init="vortex", update="FV", FB=True,
                                    xlim=(0, 10), ylim=(0, 10), BC=(("periodic", "periodic"),) * 2),
    "p2_m5_sd_lhllc": dict(p=2, m=5, N=(8, 8), init="four_quadrant", update="SD", riemann_solver_sd="lhllc",
                           BC=(("gradfree", "gradfree"),) * 2),
    "p3_ic_pressure": dict(p=3, N=(8, 8), init="four_quadrant", update="FV", FB=True, riemann_solver_sd="hllc",
                           riemann_solver_fv="hllc", BC=(("ic", "ic"), ("pressure", "pressure"))),
    # "eq" with the FV update and limiting (zero ghost subcells) turns the
    # reference's state into NaN in two steps and is refused at
    # construction; the SD update and the FV update without limiting
    # exercise the "eq" element-boundary states
    "p3_eq_1d_sd": dict(p=3, N=(16,), init="sod", update="SD", riemann_solver_sd="hllc", BC=(("eq", "eq"),)),
    "p3_eq_2d_fv_nofb": dict(p=3, N=(8, 8), init="four_quadrant", update="FV", FB=False, riemann_solver_sd="hllc",
                             BC=(("eq", "gradfree"), ("periodic", "eq"))),
    "p3_moncen_nosed_nopad": dict(p=3, N=(8, 8), init="four_quadrant", update="FV", FB=True,
                                  riemann_solver_sd="lhllc", riemann_solver_fv="llf", slope_limiter="moncen",
                                  SED=False, PAD=False, BC=(("reflective", "gradfree"), ("gradfree", "reflective"))),
    "p2_3d_delta_noblend_godunov": dict(p=2, N=(4, 4, 4), init="sedov4", update="FV", FB=True, NAD="delta",
                                        blending=False, godunov=True, riemann_solver_sd="hllc",
                                        riemann_solver_fv="hllc", BC=(("reflective", "reflective"),) * 3),
}


@pytest.mark.parametrize("name", sorted(OPTION_CASES))
def test_options_vs_oracle(name):
    """Degrees, time orders, solvers, limiters, detector switches and the
    fixed-state boundaries (ic, eq, pressure), 3 steps each, bitwise."""
    from spd_gb300 import initial_conditions as ics
    kw = dict(OPTION_CASES[name])
    init = kw.pop("init")
    kw["init_fct"] = {"four_quadrant": ics.four_quadrant, "vortex": ics.isentropic_vortex(),
                      "sod": ics.sod, "sedov4": ics.sedov(4)}[init]
    bad, _ = _run_vs_oracle(3, **kw)
    assert not bad, bad


VISC_CASES = {
    "2d_fv_nofb_gradfree_reflective": dict(p=3, N=(10, 8), init="four_quadrant", update="FV", FB=False,
                                           riemann_solver_sd="hllc", viscosity=True, nu=1e-3,
                                           BC=(("gradfree", "reflective"), ("reflective", "gradfree"))),
    "3d_sd_periodic_pressure": dict(p=2, N=(4, 5, 3), init="sedov4", update="SD", riemann_solver_sd="llf",
                                    viscosity=True, nu=2e-3, beta=0.25,
                                    BC=(("periodic", "periodic"), ("pressure", "ic"), ("reflective", "eq"))),
    "1d_sd_m2_p4": dict(p=4, m=2, N=(12,), init="sod", update="SD", riemann_solver_sd="lhllc", viscosity=True,
                        nu=1e-2, BC=(("gradfree", "gradfree"),)),
}


@pytest.mark.parametrize("name", sorted(VISC_CASES))
def test_viscosity_vs_oracle(name):
    """The viscous predictor (src/sdader_simulator.py:245-268) on further
    boundary mixes, degrees and time orders, 3 steps, bitwise."""
    from spd_gb300 import initial_conditions as ics
    kw = dict(VISC_CASES[name])
    init = kw.pop("init")
    kw["init_fct"] = {"four_quadrant": ics.four_quadrant, "sod": ics.sod, "sedov4": ics.sedov(4)}[init]
    from spd_gb300 import SDADER_Simulator
    s = SDADER_Simulator(verbose=False, **kw)
    o = oracle_like(s)
    dts = step_both(s, o, 3)
    assert all(a == b for a, b in dts), dts
    assert not compare(s, o)
    s.close()


def test_viscosity_refused_where_the_reference_fails():
    from spd_gb300 import SDADER_Simulator
    with pytest.raises(NotImplementedError, match="compute_gradient"):
        SDADER_Simulator(N=(4, 4), update="FV", FB=True, viscosity=True, verbose=False)
    s = SDADER_Simulator(N=(4, 4), update="SD", viscosity=True, verbose=False)
    with pytest.raises(Exception, match="viscous"):
        s._ctx.adjoint_enable(1)
    s.close()
