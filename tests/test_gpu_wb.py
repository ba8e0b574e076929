"""The well-balanced mode on the GPU (src/sdader_simulator.py:436-481 and
the WB branches of the step): parity with the oracle on equilibrium arrays
built by the product's own host setup, and the well-balanced property at
full size (an equilibrium initial state stays put to round-off, where the
plain scheme drifts at truncation level)."""
import numpy as np
import pytest

from gpu_helpers import compare, oracle_like, step_both

pytestmark = pytest.mark.gpu


def perturbed(base, amp=0.02):
    """``base`` with its density times 1 + amp sin(2 pi x)."""
    def f(xyz, case):
        v = base(xyz, case)
        if case == 0:
            v = v * (1.0 + amp * np.sin(2 * np.pi * xyz[0]))
        return v
    return f


WB_CASES = {
    "2d_sd_hllc_eq": dict(p=3, N=(10, 8), update="SD", riemann_solver_sd="hllc",
                          BC=(("periodic", "periodic"), ("eq", "eq"))),
    "2d_fvfb_hllc_eq": dict(p=2, N=(8, 10), update="FV", FB=True, riemann_solver_sd="hllc",
                            riemann_solver_fv="hllc", BC=(("periodic", "periodic"), ("eq", "eq")), step=True),
    "2d_fv_llf_moncen_reflective": dict(p=3, N=(8, 8), update="FV", FB=False, riemann_solver_sd="llf",
                                        riemann_solver_fv="llf", slope_limiter="moncen",
                                        BC=(("periodic", "periodic"), ("reflective", "reflective"))),
    "1d_sd_lhllc_m2": dict(p=4, m=2, N=(16,), update="SD", riemann_solver_sd="lhllc",
                           BC=(("eq", "reflective"),)),
    "1d_fvfb_llf": dict(p=3, N=(12,), update="FV", FB=True, riemann_solver_sd="llf", riemann_solver_fv="llf",
                        BC=(("eq", "eq"),)),
    "3d_sd_llf_eq": dict(p=2, N=(4, 3, 5), update="SD", riemann_solver_sd="llf",
                         BC=(("periodic", "periodic"), ("periodic", "periodic"), ("eq", "reflective"))),
    "3d_fvfb_hllc_eq": dict(p=2, N=(3, 4, 4), update="FV", FB=True, riemann_solver_sd="hllc",
                            riemann_solver_fv="hllc", BC=(("periodic", "periodic"), ("reflective", "reflective"),
                                                          ("eq", "eq")), step=True),
}


@pytest.mark.parametrize("name", sorted(WB_CASES))
def test_well_balanced_vs_oracle(name):
    """4 steps of the WB step against the oracle, bitwise, with the
    equilibrium arrays the product built (the oracle reads the same ones)."""
    from spd_gb300 import SDADER_Simulator
    from spd_gb300 import initial_conditions as ics
    kw = dict(WB_CASES[name])
    step = kw.pop("step", False)
    eq = ics.gravity_column(g=1.2, amp=0.0)
    init = ics.gravity_column(g=1.2, amp=0.05, step=True) if step else perturbed(eq)
    s = SDADER_Simulator(init_fct=init, eq_fct=eq, WB=True, potential=True, verbose=False, **kw)
    o = oracle_like(s)
    dts = step_both(s, o, 4)
    assert all(a == b for a, b in dts), dts
    assert not compare(s, o)
    s.close()


def _equilibrium_drift(n, WB, update, FB, steps):
    """Largest change of U_sp over ``steps`` steps from an atmosphere at
    rest in its gravity potential (n x n elements, p=3)."""
    from spd_gb300 import SDADER_Simulator
    from spd_gb300 import initial_conditions as ics
    eq = ics.gravity_column(amp=0.0)
    BC = (("periodic", "periodic"), ("eq", "eq") if WB or not FB else ("reflective", "reflective"))
    s = SDADER_Simulator(p=3, N=(n, n), init_fct=eq, eq_fct=eq, WB=WB, potential=True, update=update, FB=FB,
                         riemann_solver_sd="hllc", riemann_solver_fv="hllc", BC=BC, verbose=False)
    U0 = s.dm.U_sp
    s.perform_iterations(steps)
    U = s.dm.U_sp
    s.close()
    assert np.isfinite(U).all()
    return float(np.abs(U - U0).max())


@pytest.mark.parametrize("update,FB", [("SD", False), ("FV", True)])
def test_equilibrium_is_preserved_at_full_size(update, FB):
    """An atmosphere at rest in its gravity potential, 256^2 elements at
    p=3: with WB the state moves by round-off only over 20 steps."""
    assert _equilibrium_drift(256, True, update, FB, 20) < 1e-13


@pytest.mark.parametrize("update,FB", [("SD", False), ("FV", True)])
def test_equilibrium_drifts_without_well_balancing(update, FB):
    """The same atmosphere on 16^2 elements: without WB the scheme's
    truncation error moves it by orders of magnitude more than round-off
    (the contrast that shows the WB mode doing its work)."""
    wb = _equilibrium_drift(16, True, update, FB, 20)
    plain = _equilibrium_drift(16, False, update, FB, 20)
    assert wb < 1e-13 and plain > 1e3 * max(wb, 1e-16), (wb, plain)


def test_adjoint_refuses_well_balanced():
    from spd_gb300 import SDADER_Simulator
    from spd_gb300 import initial_conditions as ics
    eq = ics.gravity_column(amp=0.0)
    s = SDADER_Simulator(N=(4, 4), init_fct=eq, eq_fct=eq, WB=True, potential=True, verbose=False,
                         BC=(("periodic", "periodic"), ("eq", "eq")))
    with pytest.raises(Exception):
        s._ctx.adjoint_enable(1)
    s.close()
