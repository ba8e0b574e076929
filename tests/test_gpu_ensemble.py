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
    ens = SDADER_Ensemble(ens_sims, nstreams=nstreams, packed=False)
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
    assert steps == 6 * 2  # (packed, 1 stream, 2 streams) x 2 cpb candidates x (1 warm-up + 1 probe)
    assert len(tuning["candidates"]) == 6
    ens.perform_iterations(1)  # the chosen form keeps stepping from the probes' state
    steps += 1
    for s in ref:
        for _ in range(steps):
            s.compute_dt()
            s.perform_update()
    for a, b in zip(sims, ref):
        assert a.n_step == steps
        assert np.array_equal(a.dm.U_sp, b.dm.U_sp)
    assert tuning["form"] in ("packed", "streams") and tuning["cells_per_block"] in (16, 32)
    assert tuning["streams"] in ((None,) if tuning["form"] == "packed" else (1, 2))
    ens.close()


def _quadrant(n, p=3):
    from spd_gb300 import SDADER_Simulator
    from spd_gb300.initial_conditions import four_quadrant
    return SDADER_Simulator(p=p, N=(n, n), init_fct=four_quadrant, update="FV", FB=True,
                            riemann_solver_sd="hllc", riemann_solver_fv="hllc",
                            BC=(("gradfree", "gradfree"),) * 2, verbose=False)


def _kh_p(n, seed, p):
    from spd_gb300 import SDADER_Simulator
    from spd_gb300.initial_conditions import kelvin_helmholtz
    return SDADER_Simulator(p=p, N=(n, n), init_fct=kelvin_helmholtz(n, seed=seed), update="FV", FB=True,
                            riemann_solver_sd="hllc", riemann_solver_fv="hllc",
                            BC=(("periodic", "periodic"),) * 2, verbose=False)


def _solo_steps(sims, steps):
    for s in sims:
        for _ in range(steps):
            s.compute_dt()
            s.perform_update()


def _assert_same(ens_sims, solo, steps):
    for a, b in zip(ens_sims, solo):
        assert a.n_step == b.n_step == steps
        assert a.time == b.time
        assert np.array_equal(a.dm.U_sp, b.dm.U_sp)
        assert np.array_equal(a.dm.U_cv, b.dm.U_cv)
        assert np.array_equal(a.dm.W_cv, b.dm.W_cv)
        assert np.array_equal(a.dm.troubles, b.dm.troubles)
        assert a.dm.dt == b.dm.dt


@pytest.mark.parametrize("steps_per_launch", [1, 2])
def test_packed_ensemble_matches_individual_runs(steps_per_launch):
    """One launch per stage over all instances (block-offset table): uneven
    sides, periodic and transmissive boundaries, per-instance dt."""
    from spd_gb300 import SDADER_Ensemble
    sides = [16, 24, 8, 32, 16]
    make = [lambda i=i, n=n: _kh(n, seed=i) for i, n in enumerate(sides)] + [lambda: _quadrant(16)]
    ens_sims = [m() for m in make]
    solo = [m() for m in make]
    ens = SDADER_Ensemble(ens_sims, packed=True, steps_per_launch=steps_per_launch)
    nodes = ens.graph_nodes()
    ens.perform_iterations(4)
    _solo_steps(solo, 4)
    _assert_same(ens_sims, solo, 4)
    assert len({round(s.time, 15) for s in ens_sims}) > 1  # per-instance dt
    # the packed graph has one node per stage, however many instances
    single = SDADER_Ensemble([make[0]()], packed=True, steps_per_launch=steps_per_launch)
    assert nodes == single.graph_nodes()
    single.close()
    ens.close()


def test_packed_ensemble_odd_substeps():
    """p = 2: three FV substeps per step, so the buffer roles alternate
    between steps; several graph replays in a row."""
    from spd_gb300 import SDADER_Ensemble
    sides = [12, 20, 8]
    ens_sims = [_kh_p(n, 30 + i, 2) for i, n in enumerate(sides)]
    solo = [_kh_p(n, 30 + i, 2) for i, n in enumerate(sides)]
    ens = SDADER_Ensemble(ens_sims, packed=True)
    ens.perform_iterations(3)
    ens.perform_iterations(2)
    _solo_steps(solo, 5)
    _assert_same(ens_sims, solo, 5)
    ens.close()


def test_packed_ensemble_rejects_mixed_options():
    from spd_gb300 import SDADER_Ensemble
    from spd_gb300._lib import SpdError
    with pytest.raises(SpdError, match="degree"):
        SDADER_Ensemble([_kh_p(8, 1, 3), _kh_p(8, 2, 2)], packed=True)
    from spd_gb300 import SDADER_Simulator
    from spd_gb300.initial_conditions import kelvin_helmholtz
    no_fb = SDADER_Simulator(p=3, N=(8, 8), init_fct=kelvin_helmholtz(8, seed=3), update="FV", FB=False,
                             riemann_solver_sd="hllc", riemann_solver_fv="hllc",
                             BC=(("periodic", "periodic"),) * 2, verbose=False)
    with pytest.raises(SpdError, match="differ"):
        SDADER_Ensemble([_kh(8, seed=4), no_fb], packed=True)


@pytest.mark.parametrize("packed", [True, False])
def test_ensemble_creation_leaves_state_readable(packed):
    """Building an ensemble records one step of every instance without
    running it: the state read back before the first ensemble step is the
    state before the build (p = 2: an odd number of FV substeps, so a step
    swaps the roles of the subcell buffers)."""
    from spd_gb300 import SDADER_Ensemble
    sims = [_kh_p(n, 40 + i, 2) for i, n in enumerate([8, 16])]
    for s in sims:  # one plain step so that every buffer holds data
        s.compute_dt()
        s.perform_update()
    before = [(s.dm.U_sp, s.dm.U_cv, s.dm.W_cv, s.dm.theta) for s in sims]
    ens = SDADER_Ensemble(sims, packed=packed, nstreams=2)
    for s, (u_sp, u_cv, w_cv, theta) in zip(sims, before):
        assert np.array_equal(s.dm.U_sp, u_sp)
        assert np.array_equal(s.dm.U_cv, u_cv)
        assert np.array_equal(s.dm.W_cv, w_cv)
        assert np.array_equal(s.dm.theta, theta)
    ens.close()


@pytest.mark.parametrize("ndim", [1, 3])
def test_packed_ensemble_1d_3d(ndim):
    """Packed launches in 1D (Sod tubes, p=3) and 3D (Sedov blasts, p=2,
    reflective and transmissive walls): bit-identical to solo runs."""
    from spd_gb300 import SDADER_Ensemble, SDADER_Simulator
    from spd_gb300.initial_conditions import sedov, sod

    def make(n, bc):
        if ndim == 1:
            return SDADER_Simulator(p=3, N=(n,), init_fct=sod, update="FV", FB=True,
                                    riemann_solver_sd="hllc", riemann_solver_fv="hllc", BC=((bc, bc),),
                                    verbose=False)
        return SDADER_Simulator(p=2, N=(n, n, n), init_fct=sedov(n), update="FV", FB=True,
                                riemann_solver_sd="hllc", riemann_solver_fv="hllc", BC=((bc, bc),) * 3,
                                verbose=False)

    cases = [(64, "gradfree"), (40, "reflective"), (100, "gradfree")] if ndim == 1 else \
        [(6, "reflective"), (8, "gradfree"), (4, "reflective")]
    ens_sims = [make(n, bc) for n, bc in cases]
    solo = [make(n, bc) for n, bc in cases]
    ens = SDADER_Ensemble(ens_sims, packed=True)
    ens.perform_iterations(3)
    _solo_steps(solo, 3)
    _assert_same(ens_sims, solo, 3)
    ens.close()


def test_packed_ensemble_with_viscosity_matches_individual_runs():
    """Viscous instances (SD update, viscous dt limit active on the finer
    grids) in one packed ensemble: each instance bit-identical to stepping
    it alone."""
    from spd_gb300 import SDADER_Ensemble, SDADER_Simulator
    from spd_gb300.initial_conditions import kelvin_helmholtz

    def make(n, seed):
        return SDADER_Simulator(p=3, N=(n, n), init_fct=kelvin_helmholtz(n, seed=seed), update="SD",
                                riemann_solver_sd="hllc", viscosity=True, nu=5e-4,
                                BC=(("periodic", "periodic"),) * 2, verbose=False)

    sides = [8, 24, 16]
    ens_sims = [make(n, i) for i, n in enumerate(sides)]
    solo = [make(n, i) for i, n in enumerate(sides)]
    ens = SDADER_Ensemble(ens_sims, packed=True)
    ens.perform_iterations(3)
    for s in solo:
        for _ in range(3):
            s.compute_dt()
            s.perform_update()
    for a, b in zip(ens_sims, solo):
        assert a.time == b.time
        assert np.array_equal(a.dm.U_sp, b.dm.U_sp)
    ens.close()


@pytest.mark.parametrize("kind", ["wb_potential", "isothermal"])
def test_packed_ensemble_with_optional_physics_matches_individual_runs(kind):
    """Well-balanced gravity columns (FV with limiting, "eq" boundaries,
    equilibrium arrays per instance) and isothermal shear layers in packed
    ensembles of uneven sides: each instance bit-identical to stepping it
    alone."""
    from spd_gb300 import SDADER_Ensemble, SDADER_Simulator
    from spd_gb300 import initial_conditions as ics

    def make(n, seed):
        if kind == "wb_potential":
            eq = ics.gravity_column(amp=0.0)
            return SDADER_Simulator(p=2, N=(n, n), init_fct=ics.gravity_column(amp=0.05, step=True), eq_fct=eq,
                                    WB=True, potential=True, update="FV", FB=True, riemann_solver_sd="hllc",
                                    riemann_solver_fv="hllc", BC=(("periodic", "periodic"), ("eq", "eq")),
                                    verbose=False)
        return SDADER_Simulator(p=3, N=(n, n), init_fct=ics.kelvin_helmholtz(n, seed=seed), isothermal=True,
                                update="FV", FB=True, riemann_solver_sd="hllc", riemann_solver_fv="hllc",
                                BC=(("periodic", "periodic"),) * 2, verbose=False)

    sides = [8, 12, 16]
    ens_sims = [make(n, i) for i, n in enumerate(sides)]
    solo = [make(n, i) for i, n in enumerate(sides)]
    ens = SDADER_Ensemble(ens_sims, packed=True)
    ens.perform_iterations(3)
    _solo_steps(solo, 3)
    _assert_same(ens_sims, solo, 3)
    ens.close()
