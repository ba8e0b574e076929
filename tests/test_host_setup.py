"""Host-side setup (operators, initial state, geometry) against the
reference's outputs (CPU)."""
import os
import platform
import re

import numpy as np
import pytest

from golden_cases import DIMS, GOLDEN, case_names, golden_operators, load, make_ic
from spd_gb300.polynomials import ader_matrix
from spd_gb300.simulator import SDADER_Simulator, initial_state, subcell_faces

# NumPy's einsum/LAPACK summation orders are platform specific; the
# fixtures were made on x86_64, where the setup must match bit for bit.
EXACT = platform.machine() == "x86_64"


def same(a, b, rtol=1e-14):
    if EXACT:
        return np.array_equal(a, b)
    return np.allclose(a, b, rtol=rtol, atol=1e-15)


@pytest.mark.parametrize("p", [1, 2, 3, 4])
def test_operators_match_reference(p):
    z = np.load(os.path.join(GOLDEN, "operators.npz"))
    ops = SDADER_Simulator.build_operators(p, p)
    for key in ("x_sp", "x_fp", "sp_to_fp", "dfp_to_sp", "sp_to_cv", "x_tp", "w_tp"):
        assert same(ops[key], z[f"p{p}_{key}"]), key
    assert same(ader_matrix(ops["x_tp"], ops["w_tp"], 1.0), z[f"p{p}_ader"])


@pytest.mark.parametrize("p", range(8))
def test_point_sets_and_lagrange_rows(p):
    """Mirrors the reference's test/test_polynomials.py:9-32."""
    from spd_gb300.polynomials import flux_points, lagrange_matrix, solution_points
    tol = 1e-14
    sp = solution_points(0, 1, p)
    fp = flux_points(0, 1, p)
    assert sp.size == p + 1 and abs(2 * sp.sum() - (p + 1)) < tol and abs(sp.mean() - .5) < tol
    assert fp.size == p + 2 and abs(2 * fp.sum() - (p + 2)) < tol and abs(fp.mean() - .5) < tol
    for a in (sp, fp):
        for b in (sp, fp):
            lm = lagrange_matrix(b, a)
            assert lm.shape == (b.size, a.size)
            assert abs(lm.sum() - b.size) < tol
            assert abs(lm.mean() - 1 / a.size) < tol


@pytest.mark.parametrize("name", case_names())
def test_initial_state_matches_reference(name):
    data, kw, meta = load(name)
    ndim = len(kw["N"])
    lims = [kw.get(f"{d}lim", (0, 1)) for d in DIMS[:ndim]]
    ops = golden_operators(data)
    W_gh, W_init_cv, W_sp, U_sp, U_cv = initial_state(ndim, list(kw["N"]), kw["p"], lims, make_ic(meta["ic"]),
                                                      ops, kw.get("gamma", 1.4),
                                                      isothermal=kw.get("isothermal", False))
    assert same(W_init_cv, data["init_W_cv"])
    assert same(U_sp, data["init_U_sp"])
    assert same(U_cv, data["init_U_cv"])


def test_subcell_faces_mirror_ghosts():
    fp_ref = np.array([0.0, 0.25, 0.75, 1.0])
    f = subcell_faces(4, 0.5, fp_ref, 2)
    assert f.size == 4 * 3 + 5
    assert f[2] == 0.0 and f[-3] == 2.0
    assert np.allclose(f[:2], -f[3:5][::-1])
    assert np.all(np.diff(f) > 0)


def test_unsupported_options_raise():
    for kw in ({"viscosity": True, "update": "FV", "FB": True}, {"predictor": False}, {"p": 0}, {"p": 5}):
        with pytest.raises(NotImplementedError):
            SDADER_Simulator(N=(4,), **kw)
    with pytest.raises(AttributeError):
        SDADER_Simulator(N=(4,), riemann_solver_sd="roe")
    with pytest.raises(AttributeError):
        SDADER_Simulator(N=(4,), slope_limiter="superbee")
    with pytest.raises(TypeError):
        SDADER_Simulator(N=(4,), BC=(("open", "open"),))
    # "eq" boundaries with the FV update and limiting: the reference's state
    # becomes NaN in two steps (zero-density ghost subcells); refused
    with pytest.raises(NotImplementedError, match="eq"):
        SDADER_Simulator(N=(4, 4), update="FV", FB=True, BC=(("eq", "gradfree"), ("periodic", "periodic")))


@pytest.mark.parametrize("ndim,p,N", [(1, 3, 3000), (2, 3, 40), (2, 2, 96), (3, 2, 20), (3, 4, 12)])
def test_threaded_transform_full_is_bitwise(ndim, p, N):
    """transform_full on thread slabs gives the same bits as one einsum."""
    from spd_gb300.polynomials import transform_full, transform_full_threaded
    rng = np.random.default_rng(ndim * 100 + p)
    shape = (ndim + 2,) + (N,) * ndim + (p + 1,) * ndim
    B = rng.standard_normal(shape) * 10.0 ** rng.uniform(-6, 6, shape)
    A = SDADER_Simulator.build_operators(p, p)["cv_to_sp"]
    assert np.array_equal(transform_full(B, A, ndim), transform_full_threaded(B, A, ndim, min_cells=1, workers=4))


def test_initial_state_builds_quadrature_points_once():
    """initial_state (points built once, threaded transform) equals the
    per-variable quadrature and single-call transform of the reference."""
    from spd_gb300.initial_conditions import kelvin_helmholtz
    from spd_gb300.polynomials import quadrature_mean, transform_full
    from spd_gb300.simulator import mesh_cv
    N, p = [300, 260], 3
    ops = SDADER_Simulator.build_operators(p, p)
    fct = kelvin_helmholtz(300, seed=5)
    W_gh, W_init_cv, W_sp, U_sp, U_cv = initial_state(2, N, p, [(0.0, 1.0), (0.0, 1.0)], fct, ops, 1.4)
    mesh = mesh_cv(2, N, p, [(0.0, 1.0), (0.0, 1.0)], 1, ops["x_fp"])
    for var in range(4):
        assert np.array_equal(W_gh[var], quadrature_mean(mesh, fct, 2, var))
    assert np.array_equal(W_sp, transform_full(W_init_cv.copy(), ops["cv_to_sp"], 2))


@pytest.mark.parametrize("ndim,p,N", [(1, 3, 4000), (2, 3, 150), (2, 2, 97), (3, 2, 24), (3, 3, 13)])
def test_threaded_quadrature_is_bitwise(ndim, p, N):
    """Quadrature points and per-variable cell means on thread slabs give
    the same bits as the single-threaded forms."""
    from spd_gb300.initial_conditions import four_quadrant, kelvin_helmholtz, sedov, sod
    from spd_gb300.polynomials import quadrature_mean, quadrature_points, quadrature_points_threaded
    from spd_gb300.simulator import mesh_cv
    fct = {1: sod, 2: kelvin_helmholtz(N, seed=2) if p == 3 else four_quadrant, 3: sedov(N)}[ndim]
    ops = SDADER_Simulator.build_operators(p, p)
    mesh = mesh_cv(ndim, [N] * ndim, p, [(0.0, 1.0)] * ndim, 1, ops["x_fp"])
    a, wa = quadrature_points(mesh, ndim)
    b, wb = quadrature_points_threaded(mesh, ndim, workers=4, min_cells=1)
    assert np.array_equal(a, b) and np.array_equal(wa, wb) and not b.flags.writeable
    for v in range(ndim + 2):
        assert np.array_equal(quadrature_mean(mesh, fct, ndim, v, points=(a, wa)),
                              quadrature_mean(mesh, fct, ndim, v, points=(b, wb), workers=4))
