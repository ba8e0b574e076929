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
                                                      ops, kw.get("gamma", 1.4))
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
    for kw in ({"viscosity": True}, {"potential": True}, {"WB": True}, {"isothermal": True},
               {"predictor": False}):
        with pytest.raises(NotImplementedError):
            SDADER_Simulator(N=(4,), **kw)
    with pytest.raises(AttributeError):
        SDADER_Simulator(N=(4,), riemann_solver_sd="roe")
    with pytest.raises(AttributeError):
        SDADER_Simulator(N=(4,), slope_limiter="superbee")
    with pytest.raises(TypeError):
        SDADER_Simulator(N=(4,), BC=(("open", "open"),))
