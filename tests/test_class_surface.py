"""The reference's class surface on the host (CPU): the constructor chain
SDADER_Simulator -> SD_Simulator -> FV_Simulator -> Simulator binds the
same positional and keyword arguments, the base classes build without a
device as the reference's do (its test/test_create.py:12-16 creates all
four), and the array-shape helpers return the reference's shapes."""
import numpy as np
import pytest

from spd_gb300 import FV_Simulator, SDADER_Simulator, SD_Simulator, Simulator


@pytest.mark.parametrize("p", [1, 3])
@pytest.mark.parametrize("N", [(6,), (6, 6), (6, 6, 6)])
@pytest.mark.parametrize("cls", [Simulator, FV_Simulator])
def test_create_host_classes(p, N, cls):
    s = cls(p=p, N=N, use_cupy=False)
    assert s.nvar == len(N) + 2 and s._p_ == len(N) + 1
    assert list(s.vels) == list(range(1, len(N) + 1))
    assert s.h_min == pytest.approx(1 / 6)


def test_class_chain_and_bases():
    assert SDADER_Simulator.__mro__[1:4] == (SD_Simulator, FV_Simulator, Simulator)
    assert issubclass(SD_Simulator, Simulator) and not issubclass(SD_Simulator, FV_Simulator)


def test_fv_options_are_checked_on_the_fv_class():
    with pytest.raises(AttributeError):
        FV_Simulator(N=(4,), riemann_solver_fv="roe")
    with pytest.raises(AttributeError):
        FV_Simulator(N=(4,), slope_limiter="superbee")
    f = FV_Simulator("hllc", "moncen", True, None, None, 2, -1, (4, 4))  # positional, as the reference binds
    assert (f.riemann_solver_fv_name, f.slope_limiter_name, f.p, f.N["y"]) == ("hllc", "moncen", 2, 4)


def test_unknown_keyword_is_a_type_error():
    with pytest.raises(TypeError):
        SDADER_Simulator(N=(4,), bogus=1)


def test_fv_array_shapes():
    f = FV_Simulator(p=3, N=(6, 5))
    # src/fv_simulator.py:24-37: one value per cell
    assert f.array_FV(4, dim="x", ngh=2).shape == (4, 9, 11)
    assert f.array_FV(1).shape == (1, 5, 6)
    assert f.array_FV_BC("y").shape == (2, 4, 2, 10)


def test_sd_array_shapes_without_a_device():
    """array_fp / array_RS / array_BC / array_FV(n, ...) of
    src/sd_simulator.py:133-182 and src/sdader_simulator.py:273-286, on an
    object whose device context is never created."""
    s = object.__new__(SDADER_Simulator)
    Simulator.__init__(s, p=3, N=(6, 5, 4))
    s.n = {d: 4 for d in s.dims}
    s.nader = 4
    assert s.array_sp().shape == (5, 4, 5, 6, 4, 4, 4)
    assert s.array_fp(dims="y", ader=True).shape == (5, 4, 4, 5, 6, 4, 5, 4)
    assert s.array_fp().shape == (5, 4, 5, 6, 5, 5, 5)
    assert s.array_RS(dim="x", ader=True).shape == (5, 4, 4, 5, 7, 4, 4)
    assert s.array_RS(dim="z").shape == (5, 5, 5, 6, 4, 4)
    assert s.array_BC(dim="x", ader=True).shape == (2, 5, 4, 4, 5, 4, 4)
    assert s.array_BC(dim="y").shape == (2, 5, 4, 6, 4, 4)
    assert s.array_BC(dim="z").shape == (2, 5, 5, 6, 4, 4)
    assert s.array_FV(4, 1, dim="z", ngh=0).shape == (1, 17, 20, 24)
    assert s.array_FV_BC("x").shape == (2, 5, 20, 24, 2)


def test_integrate_faces_averages_the_other_directions():
    """Constant data stays constant under the transverse subcell average
    (the rows of sp_to_cv sum to one)."""
    s = object.__new__(SDADER_Simulator)
    Simulator.__init__(s, p=2, N=(3, 2))
    s.ops = SDADER_Simulator.build_operators(2, 2)
    M = np.full((4, 3, 2, 3, 3, 4), 2.5)  # (V, T, Ny, Nx, ny, nx+1): x flux points
    out = s.integrate_faces(M, "x")
    assert out.shape == M.shape
    assert np.allclose(out, 2.5, rtol=0, atol=1e-14)


@pytest.mark.parametrize("name", ["pot_column8_p2_sd_hllc_reflective", "pot_column4_p2_fv_llf_3d",
                                  "pot_visc_column16_p3_sd_llf_1d"])
def test_potential_gradients_match_reference(name):
    """init_potential (src/sdader_simulator.py:425-434) on the host: the
    gradient at the solution points and its subcell averages equal the
    reference's, bit for bit (x86_64, where the fixtures were made)."""
    import platform
    from golden_cases import load, make_ic
    from spd_gb300.simulator import mesh_cv
    data, kw, meta = load(name)
    s = object.__new__(SDADER_Simulator)
    Simulator.__init__(s, p=kw["p"], N=kw["N"], init_fct=make_ic(meta["ic"]),
                       **{k: kw[k] for k in ("xlim", "ylim", "zlim") if k in kw})
    s.ops = SDADER_Simulator.build_operators(kw["p"], kw["p"])
    s.n = {d: kw["p"] + 1 for d in s.dims}
    s.nader = kw["p"] + 1
    s.fp = {d: s.ops["x_fp"] for d in s.dims}
    s.mesh_cv = mesh_cv(s.ndim, [s.N[d] for d in s.dims], s.p, [s.lim[d] for d in s.dims], s.Nghe, s.ops["x_fp"])
    s.potential = True
    s.init_potential()
    same = platform.machine() in ("x86_64", "AMD64")
    for key in ("grad_phi_sp", "grad_phi_fv"):
        got, want = getattr(s.dm, key), data[key]
        assert got.shape == want.shape
        if same:
            assert np.array_equal(got, want), key
        else:
            assert np.allclose(got, want, rtol=1e-13, atol=1e-13), key
