"""Batched ensemble of uneven grids: every instance bit-identical to
stepping it alone, per-instance dt."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _kh(n, seed):
    from spd_gb300 import SDADER_Simulator
    from spd_gb300.initial_conditions import kelvin_helmholtz
    return SDADER_Simulator(p=3, N=(n, n), init_fct=kelvin_helmholtz(n, seed=seed), update="FV", FB=True,
                            riemann_solver_sd="hllc", riemann_solver_fv="hllc",
                            BC=(("periodic", "periodic"),) * 2, verbose=False)


@pytest.mark.parametrize("nstreams", [1, 3])
def test_ensemble_matches_individual_runs(nstreams):
    from spd_gb300 import SDADER_Ensemble
    sides = [16, 24, 8, 32, 16]
    ens_sims = [_kh(n, seed=i) for i, n in enumerate(sides)]
    solo = [_kh(n, seed=i) for i, n in enumerate(sides)]
    ens = SDADER_Ensemble(ens_sims, nstreams=nstreams)
    ens.perform_iterations(4)
    for s in solo:
        for _ in range(4):
            s.compute_dt()
            s.perform_update()
    for a, b in zip(ens_sims, solo):
        assert a.n_step == b.n_step == 4
        assert a.time == b.time
        assert np.array_equal(a.dm.U_sp, b.dm.U_sp)
        assert np.array_equal(a.dm.W_cv, b.dm.W_cv)
        assert np.array_equal(a.dm.troubles, b.dm.troubles)
    dts = {round(s.time, 15) for s in ens_sims}
    assert len(dts) > 1  # per-instance dt
    ens.close()


def test_ensemble_autotune_keeps_results():
    from spd_gb300 import SDADER_Ensemble
    sims = [_kh(n, seed=7 + i) for i, n in enumerate([8, 16])]
    ref = [_kh(n, seed=7 + i) for i, n in enumerate([8, 16])]
    ens = SDADER_Ensemble(sims)
    tuning = ens.autotune(streams=(1, 2), cpbs=(16, 32), probe_launches=1)
    steps = sims[0].n_step
    assert steps == 4 * 2  # 4 candidates x (1 warm-up + 1 probe)
    for s in ref:
        for _ in range(steps):
            s.compute_dt()
            s.perform_update()
    for a, b in zip(sims, ref):
        assert np.array_equal(a.dm.U_sp, b.dm.U_sp)
    assert tuning["streams"] in (1, 2) and tuning["cells_per_block"] in (16, 32)
    ens.close()
