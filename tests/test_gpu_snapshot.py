"""State snapshots: a run saved after k steps and restored into a fresh
simulator continues bit for bit like the uninterrupted run."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("update", ["FV", "SD"])
def test_snapshot_resume_is_bitwise(tmp_path, update):
    from spd_gb300 import SDADER_Simulator
    from spd_gb300.initial_conditions import four_quadrant
    kw = dict(p=3, N=(32, 32), init_fct=four_quadrant, update=update, FB=(update == "FV"),
              riemann_solver_sd="hllc", riemann_solver_fv="hllc", BC=(("gradfree", "gradfree"),) * 2,
              verbose=False)
    a = SDADER_Simulator(**kw)
    for _ in range(10):
        a.compute_dt()
        a.perform_update()
    b = SDADER_Simulator(**kw)
    for _ in range(4):
        b.compute_dt()
        b.perform_update()
    path = tmp_path / "state.npz"
    b.save_state(path)
    b.close()
    c = SDADER_Simulator(**kw)
    c.restore_state(path)
    assert c.n_step == 4
    for _ in range(6):
        c.compute_dt()
        c.perform_update()
    assert c.time == a.time and c.n_step == a.n_step
    for key in ("U_sp", "U_cv", "W_cv"):
        assert np.array_equal(getattr(a.dm, key), getattr(c.dm, key)), key
    a.close()
    c.close()


def test_snapshot_rejects_another_configuration(tmp_path):
    from spd_gb300 import SDADER_Simulator
    a = SDADER_Simulator(p=2, N=(8, 8), verbose=False)
    a.save_state(tmp_path / "s.npz")
    b = SDADER_Simulator(p=3, N=(8, 8), verbose=False)
    with pytest.raises(ValueError):
        b.restore_state(tmp_path / "s.npz")
    a.close()
    b.close()
