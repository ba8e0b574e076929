"""The opt-in build with fused multiply-adds (SDADER_Simulator(fma=True)):
not bit-identical to the reference, so it is held to the specification's
tolerances against the product build (which is): normwise relative
difference of U_sp per variable <= 1e-12 after one step and <= 1e-10 after
100 steps, on the isentropic vortex (32x32, p=3, FV with limiting, LLF; the
limiter stays inactive, so the trouble masks are identical)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _normrel(a, b):
    return max(float(np.max(np.abs(a[v] - b[v])) / np.max(np.abs(b[v]))) for v in range(b.shape[0]))


def test_fma_build_within_tolerance_on_the_vortex():
    from spd_gb300 import SDADER_Simulator
    from spd_gb300.initial_conditions import isentropic_vortex
    kw = dict(p=3, N=(32, 32), xlim=(0, 10), ylim=(0, 10), init_fct=isentropic_vortex(), update="FV", FB=True,
              riemann_solver_sd="llf", riemann_solver_fv="llf", BC=(("periodic", "periodic"),) * 2, verbose=False)
    a = SDADER_Simulator(**kw)
    f = SDADER_Simulator(fma=True, **kw)
    assert f._ctx.variant == "fma" and a._ctx.variant == "ieee"
    for k in range(100):
        a.compute_dt()
        f.compute_dt()
        a.perform_update()
        f.perform_update()
        assert np.array_equal(a.dm.troubles, f.dm.troubles)
        if k == 0:
            d1 = _normrel(f.dm.U_sp, a.dm.U_sp)
            assert 0.0 < d1 <= 1e-12, d1  # a different build: not bitwise, within 1e-12
    d100 = _normrel(f.dm.U_sp, a.dm.U_sp)
    assert d100 <= 1e-10, d100
    a.close()
    f.close()


def test_fma_and_product_contexts_coexist_in_one_process():
    """Both libraries load side by side; an ensemble refuses to mix them."""
    from spd_gb300 import SDADER_Ensemble, SDADER_Simulator
    from spd_gb300.initial_conditions import four_quadrant
    kw = dict(p=2, N=(8, 8), init_fct=four_quadrant, update="FV", FB=True, BC=(("gradfree", "gradfree"),) * 2,
              verbose=False)
    a = SDADER_Simulator(**kw)
    f = SDADER_Simulator(fma=True, **kw)
    with pytest.raises(ValueError, match="one library"):
        SDADER_Ensemble([a, f])
    e = SDADER_Ensemble([f, SDADER_Simulator(fma=True, **kw)])
    e.perform_iterations(2)
    e.close()
    a.close()
    f.close()
