"""Drop-in ``SDADER_Simulator`` whose time step runs on the GPU.

The class keeps the constructor, the step/run methods, the state arrays
(``s.dm.U_sp`` etc., reference layouts) and the options of the reference's
SDADER_Simulator (src/sdader_simulator.py:14-476 with its bases
src/sd_simulator.py:19-239, src/fv_simulator.py:10-285,
src/simulator.py:9-209).  Setup (operators, positions, initial
condition quadrature) is host NumPy as in the reference; every step runs in
the CUDA library through spd_gb300._lib.  There is no CPU path for the
step.
"""
from __future__ import annotations

import ctypes
import os
from collections import defaultdict
from timeit import default_timer as timer
from typing import Callable, Tuple

import warnings

import numpy as np

from . import _lib
from .initial_conditions import sine_wave
from .polynomials import (ader_matrix, flux_points, gauss_legendre_quadrature, intfromsol_matrix,
                          lagrange_matrix, lagrangeprime_matrix, quadrature_mean, quadrature_points_threaded,
                          solution_points, transform_axis, transform_full, transform_full_threaded)

DIMS = ("x", "y", "z")


def _primitives(U, vels, _p_, gamma, isothermal=False):
    """src/hydro.py:48-86 on the host (user-facing helper)."""
    W = U.copy()
    K = W[0].copy() * 0
    for vel in vels:
        W[vel] = U[vel] / U[0]
        K += W[vel] ** 2
    K *= 0.5 * U[0]
    K *= 0 if isothermal else 1
    W[_p_] = (gamma - 1) * (U[_p_] - K)
    return W


def _fluxes(W, vels, _p_, gamma, isothermal=False):
    """src/hydro.py:127-170 on the host (setup of the well-balanced mode):
    the Euler flux in the rotated frame ``vels``."""
    F = W.copy()
    v1 = vels[0]
    K = W[0].copy() * 0
    m = None
    for v in vels[::-1]:
        m = W[0] * W[v]
        K += m * W[v]
        F[v, ...] = m * W[v1]
    E = W[_p_] / (gamma - 1) + 0.5 * K
    F[0, ...] = m
    F[v1, ...] = m * W[v1] + W[_p_]
    F[_p_, ...] = W[v1] * (E + W[_p_])
    F[_p_, ...] *= 0 if isothermal else 1
    return F


def _crop_fv(start, end, idim, ndim, ngh):
    """src/slicing.py:27-31."""
    return (Ellipsis,) + (slice(ngh, -ngh),) * (ndim - 1 - idim) + (slice(start, end),) + (slice(ngh, -ngh),) * idim


def _conservatives(W, vels, _p_, gamma, isothermal=False):
    """src/hydro.py:88-125 on the host (setup and user-facing helper)."""
    U = W.copy()
    K = W[0].copy() * 0
    for vel in vels:
        U[vel] = W[vel] * U[0]
        K += W[vel] ** 2
    K *= 0.5 * U[0]
    K *= 0 if isothermal else 1
    U[_p_] = W[_p_] / (gamma - 1) + K
    return U


def mesh_cv(ndim, N, p, lims, Nghe, fp_ref) -> np.ndarray:
    """Flux-point coordinates of every cell including Nghe ghost layers,
    shape (ndim, [Nz,] [Ny,] Nx, p+2, ...) (src/sd_simulator.py:59-72)."""
    Ns = [N[i] + 2 * Nghe for i in range(ndim)]
    shape = (ndim,) + tuple(Ns[::-1]) + (p + 2,) * ndim
    mesh = np.ndarray(shape)
    for idim in range(ndim):
        Nd = Ns[idim]
        h = (lims[idim][1] - lims[idim][0]) / N[idim]
        length = (lims[idim][1] - lims[idim][0]) + 2 * Nghe * h
        s1 = (None,) * (ndim - 1 - idim) + (slice(None),) + (None,) * (ndim + idim)
        s2 = (None,) * (2 * ndim - 1 - idim) + (slice(None),) + (None,) * idim
        mesh[idim] = lims[idim][0] + (np.arange(Nd)[s1] + fp_ref[s2]) * length / Nd - h
    return mesh


def subcell_faces(N, h, fp_ref, ngh) -> np.ndarray:
    """Subcell face positions of one direction with ngh mirrored ghost faces
    per side (src/sdader_simulator.py:73-78)."""
    n = len(fp_ref) - 1
    fp = np.ndarray(N * n + ngh * 2 + 1)
    fp[ngh:-ngh] = h * np.hstack((np.arange(N).repeat(n) + np.tile(fp_ref[:-1], N), N))
    fp[:ngh] = -fp[(ngh + 1):(2 * ngh + 1)][::-1]
    fp[-ngh:] = fp[-(ngh + 1)] + fp[ngh + 1:2 * ngh + 1]
    return fp


def initial_state(ndim, N, p, lims, init_fct, ops, gamma, Nghe=1, isothermal=False):
    """Initial subcell averages of the primitives and the derived
    solution-point / conservative arrays (src/sd_simulator.py:74-90).
    Returns (W_gh, W_init_cv, W_sp, U_sp, U_cv)."""
    nvar = ndim + 2
    vels = np.arange(ndim) + 1
    mesh = mesh_cv(ndim, N, p, lims, Nghe, ops["x_fp"])
    W_gh = np.ndarray((nvar,) + tuple(N[i] + 2 * Nghe for i in range(ndim))[::-1] + (p + 1,) * ndim)
    # the quadrature points are the same for every variable: built once;
    # large grids build them and sum each variable on host thread slabs
    ncells = int(np.prod([N[i] + 2 * Nghe for i in range(ndim)]))
    workers = min(16, os.cpu_count() or 1) if ncells >= (1 << 15) else 1
    points = quadrature_points_threaded(mesh, ndim, workers=workers)
    for var in range(nvar):
        W_gh[var] = quadrature_mean(mesh, init_fct, ndim, var, points=points, workers=workers)
    del points
    W_init_cv = W_gh[(slice(None),) + (slice(Nghe, -Nghe),) * ndim + (Ellipsis,)]
    W_cv = W_init_cv.copy()
    W_sp = transform_full_threaded(W_cv, ops["cv_to_sp"], ndim)
    U_sp = _conservatives(W_sp, vels, ndim + 1, gamma, isothermal)
    U_cv = _conservatives(W_cv, vels, ndim + 1, gamma, isothermal)
    return W_gh, W_init_cv, W_sp, U_sp, U_cv


class _DataManager:
    """Stand-in for the reference's GPUDataManager (src/data_management.py:
    32-68): device-resident fields are downloaded on read (a fresh NumPy
    array) and uploaded on assignment; constants live on the host."""

    _device_fields = ("U_sp", "U_cv", "W_cv", "troubles", "theta",
                      "affected_faces_x", "affected_faces_y", "affected_faces_z")

    def __init__(self, sim):
        object.__setattr__(self, "_sim", sim)
        object.__setattr__(self, "_host", {})

    @property
    def xp(self):
        return np

    def switch_to(self, location):
        return None

    def asnumpy(self, arr):
        return np.asarray(arr)

    def __getattr__(self, name):
        sim = object.__getattribute__(self, "_sim")
        if name == "dt":
            return sim._ctx.get_dt()
        if name in _DataManager._device_fields and sim._ctx is not None:
            return sim._download(name)
        host = object.__getattribute__(self, "_host")
        if name.startswith("F_ader_fp_") and name not in host and sim._ctx is not None:
            return sim._F_ader_fp(name[-1])
        if name in host:
            return host[name]
        raise AttributeError(name)

    def __setattr__(self, name, value):
        sim = object.__getattribute__(self, "_sim")
        if name == "dt" and sim._ctx is not None:
            sim._ctx.set_dt(float(value))
            return
        if name in ("U_sp", "U_cv", "W_cv") and sim._ctx is not None:
            sim._ctx.upload(name, np.asarray(value, dtype=np.float64))
            return
        if name in ("grad_phi_sp", "grad_phi_fv") and sim._ctx is not None and sim.potential:
            # the gravity gradients: at the solution points (SD layout) and
            # their subcell averages (FV layout, sent in the SD layout)
            value = np.ascontiguousarray(value, dtype=np.float64)
            if name == "grad_phi_sp":
                sim._ctx.upload("grad_phi_sp", value)
            else:
                sim._ctx.upload("grad_phi_cv", np.ascontiguousarray(sim.transpose_to_sd(value)))
        object.__getattribute__(self, "_host")[name] = value


class Simulator:
    """Base of the simulator classes (src/simulator.py:9-209): geometry,
    variable indices, options and the host-side layout helpers.  It holds no
    device state, as the reference's base class holds no step."""

    def __init__(self,
                 init_fct: Callable = sine_wave,
                 eq_fct: Callable = sine_wave,
                 p: int = 1,
                 m: int = -1,
                 N: Tuple = (32, 32),
                 Nghe: int = 1,
                 Nghc: int = 2,
                 xlim: Tuple = (0, 1),
                 ylim: Tuple = (0, 1),
                 zlim: Tuple = (0, 1),
                 gamma: float = 1.4,
                 beta: float = 2. / 3,
                 nu: float = 1e-4,
                 cfl_coeff: float = 0.8,
                 min_c2: float = 1E-10,
                 isothermal: bool = False,
                 viscosity: bool = False,
                 potential: bool = False,
                 WB: bool = False,
                 use_cupy: bool = True,
                 BC: Tuple = (("periodic", "periodic"),
                              ("periodic", "periodic"),
                              ("periodic", "periodic")),
                 verbose=True):
        if not hasattr(self, "_ctx"):
            self._ctx = None
        # ---- src/simulator.py:37-126 ----------------------------------
        self.init_fct = init_fct
        self.eq_fct = eq_fct
        if m == -1:
            m = p
        self.p = p
        self.m = m
        ndim = len(N)
        self.ndim = ndim
        assert len(BC) >= ndim
        self.BC = {}
        self.idims = {}
        self.dims = {}
        for idim in range(ndim):
            dim = DIMS[idim]
            self.idims[idim] = dim
            self.dims[dim] = idim
            self.BC[dim] = BC[idim]
            for side in (0, 1):
                if BC[idim][side] not in _lib.BCKIND:
                    raise TypeError("Undetermined boundary type")
            setattr(self, f"N{dim}", N[idim])
        self.Y = ndim > 1
        self.Z = ndim > 2
        self.xlim, self.ylim, self.zlim = xlim, ylim, zlim
        self.time = 0.0
        self.Nghe = Nghe
        self.Nghc = Nghc
        self.gamma = gamma
        self.beta = beta
        self.nu = nu
        self.cfl_coeff = cfl_coeff
        self.min_c2 = min_c2
        self.isothermal = isothermal
        self.viscosity = viscosity
        self.potential = potential
        self.WB = WB
        self.verbose = verbose
        self.use_cupy = use_cupy
        self.dm = _DataManager(self)
        self.nghx = Nghc
        self.nghy = (0, Nghc)[self.Y]
        self.nghz = (0, Nghc)[self.Z]
        self.lim, self.len, self.h, self.N, self.ngh = {}, {}, {}, {}, {}
        self.h_min = 1E10
        for dim in self.dims:
            self.lim[dim] = getattr(self, f"{dim}lim")
            setattr(self, f"{dim}len", self.lim[dim][1] - self.lim[dim][0])
            self.len[dim] = getattr(self, f"{dim}len")
            self.N[dim] = getattr(self, f"N{dim}")
            setattr(self, f"d{dim}", self.len[dim] / self.N[dim])
            self.h[dim] = getattr(self, f"d{dim}")
            self.ngh[dim] = getattr(self, f"ngh{dim}")
            self.h_min = min(self.h_min, self.h[dim])
        self.n_step = 0
        self.variables = [r"$\rho$"]
        self._d_ = 0
        self.vels = np.arange(ndim) + 1
        for dim in self.dims:
            name = f"v{dim}"
            self.variables.append(name)
            setattr(self, f"_{name}_", self.vels[self.dims[dim]])
        self.variables.append("P")
        self._p_ = ndim + 1
        self.nvar = ndim + 2
        self.rank = 0

    def shape(self, idim):
        return (None,) * (self.ndim - idim) + (slice(None),) + (None,) * idim

    def domain_size(self):
        return [self.N[dim] * self.n[dim] for dim in self.dims]

    def regular_faces(self):
        return [np.linspace(self.lim[dim][0], self.lim[dim][1], self.N[dim] * self.n[dim] + 1) for dim in self.dims]

    def regular_centers(self):
        return [np.linspace(self.lim[dim][0], self.lim[dim][1], self.N[dim] * self.n[dim]) for dim in self.dims]

    def crop(self, M, ngh=1) -> np.ndarray:
        return M[(slice(None),) + (slice(ngh, -ngh),) * self.ndim + (Ellipsis,)]

    def compute_primitives(self, U, **kwargs) -> np.ndarray:
        return _primitives(U, self.vels, self._p_, self.gamma, self.isothermal)

    def compute_conservatives(self, W, **kwargs) -> np.ndarray:
        return _conservatives(W, self.vels, self._p_, self.gamma, self.isothermal)

    def compute_positions(self):
        pass

    def compute_mesh_cv(self):
        pass

    def post_init(self):
        pass

    def compute_dt(self) -> None:
        pass


class FV_Simulator(Simulator):
    """The finite-volume base class (src/fv_simulator.py:10-285): Riemann
    solver, slope limiter and predictor options and the subcell array
    shapes.  Like the reference's, it holds no step of its own; the
    subcell update runs inside SDADER_Simulator's step on the GPU."""

    def __init__(self, riemann_solver_fv: str = "llf", slope_limiter: str = "minmod", predictor: bool = True,
                 *args, **kwargs):
        super().__init__(*args, **kwargs)
        if riemann_solver_fv not in _lib.RIEMANN:
            raise AttributeError(riemann_solver_fv)
        if slope_limiter not in _lib.LIMITER:
            raise AttributeError(slope_limiter)
        self.riemann_solver_fv_name = riemann_solver_fv
        self.slope_limiter_name = slope_limiter
        self.predictor = predictor

    def array_FV(self, nvar, dim=None, ngh=0) -> np.ndarray:
        """src/fv_simulator.py:24-29 (one value per cell)."""
        N = [self.N[d2] + (dim == d2) + 2 * ngh for d2 in self.dims]
        return np.ndarray([nvar] + N[::-1])

    def array_FV_BC(self, dim="x") -> np.ndarray:
        """src/fv_simulator.py:31-37."""
        ngh = self.Nghc
        N = [self.N[d2] + 2 * ngh if dim != d2 else ngh for d2 in self.dims]
        return np.ndarray([2, self.nvar] + N[::-1])


class SD_Simulator(Simulator):
    """The spectral-difference class (src/sd_simulator.py:19-239): constant
    operators, mesh, initial state and the CFL dt, with the state on the
    GPU.  Constructed on its own it steps with the SD update and no
    limiter; SDADER_Simulator (its subclass) adds the options of the
    reference's SDADER class.  Options the GPU step does not implement
    (predictor=False, and viscosity with the FV update and FB, which fails
    in the reference itself) raise NotImplementedError here, before any
    device work.
    """

    def __init__(self, riemann_solver_sd: str = "llf", update: str = "SD", *args, **kwargs):
        super().__init__(*args, **kwargs)
        # options of the classes below SD_Simulator in the reference's chain
        # (FV_Simulator, SDADER_Simulator), at their defaults when absent
        for key, val in (("riemann_solver_fv_name", "llf"), ("slope_limiter_name", "minmod"), ("predictor", True),
                         ("FB", False), ("tolerance", 1e-5), ("SED", True), ("NAD", ""), ("PAD", True),
                         ("blending", True), ("min_rho", 1e-10), ("max_rho", 1e10), ("min_P", 1e-10),
                         ("godunov", False), ("fma", False), ("_operators", None)):
            if not hasattr(self, key):
                setattr(self, key, val)
        if not self.predictor:
            raise NotImplementedError("predictor=False (plain MUSCL) is not implemented "
                                      "(the reference's path raises AttributeError)")
        if self.Nghc != 2:
            raise NotImplementedError("only Nghc=2 subcell ghost layers are supported")
        if not 1 <= self.p <= 4:
            raise NotImplementedError(f"p={self.p}: the kernels are instantiated for degrees 1 to 4")
        if riemann_solver_sd not in _lib.RIEMANN:
            raise AttributeError(riemann_solver_sd)
        if update not in _lib.UPDATE:
            raise ValueError(f"update must be 'SD' or 'FV', got {update!r}")
        if update == "FV" and self.FB and not self.WB and any(side == "eq" for d in self.dims for side in self.BC[d]):
            # src/fv_simulator.py:251-253 fills "eq" ghost subcells with zeros
            # (the perturbation of the well-balanced mode, not implemented
            # here); the reference's MUSCL-Hancock fluxes at those faces are
            # then NaN, and theta*F_FB + (1-theta)*F_HO turns the boundary
            # cells into NaN in the first step and every cell in the second
            raise NotImplementedError(
                "BC 'eq' with update='FV', FB=True and WB=False: the reference's fallback fluxes at those "
                "boundaries are NaN (zero-density ghost subcells outside well-balanced mode), so its state becomes "
                "NaN in the first two steps; this combination is refused instead of reproducing a NaN state")
        if self.viscosity and update == "FV" and self.FB:
            # src/fv_simulator.py:186-187 -> src/muscl.py:253 -> src/fv_simulator.py:74
            # -> src/muscl.py:97 calls Slope_limiter.compute_gradient, which does
            # not exist: the reference's first step with these options raises
            raise NotImplementedError(
                "viscosity=True with update='FV' and FB=True: the reference's viscous fallback fluxes raise "
                "AttributeError ('Slope_limiter' object has no attribute 'compute_gradient'); viscosity runs with "
                "the SD update or the FV update without FB")
        self.riemann_solver_sd_name = riemann_solver_sd
        self.update = update
        p, m, ndim = self.p, self.m, self.ndim
        # ---- SD_Simulator operators (src/sd_simulator.py:30-52) ------------
        self.x, self.w = gauss_legendre_quadrature(0.0, 1.0, p)
        sp = solution_points(0.0, 1.0, p)
        fp = flux_points(0.0, 1.0, p)
        self.sp, self.fp, self.n = defaultdict(list), defaultdict(list), defaultdict(list)
        for dim in self.dims:
            setattr(self, f"{dim}_sp", sp)
            self.sp[dim] = sp
            setattr(self, f"{dim}_fp", fp)
            self.fp[dim] = fp
            setattr(self, f"n{dim}", p + 1)
            self.n[dim] = p + 1
        operators = self._operators if self._operators is not None else self.build_operators(p, m)
        self.ops = operators
        for key in ("sp_to_fp", "fp_to_sp", "dfp_to_sp", "sp_to_cv", "fp_to_cv", "cv_to_sp",
                    "x_tp", "w_tp", "invader"):
            if key in operators:
                setattr(self.dm, key, operators[key])
        self.nader = m + 1
        # ---- geometry and initial state (src/sd_simulator.py:59-90) ----
        self.mesh_cv = self.compute_mesh_cv()
        self.compute_positions()
        W_gh, self.W_init_cv, W_sp, U_sp, U_cv = initial_state(
            ndim, [self.N[d] for d in self.dims], p, [self.lim[d] for d in self.dims], self.init_fct,
            operators, self.gamma, self.Nghe, self.isothermal)
        W_cv = self.W_init_cv.copy()
        self.dm.W_sp = W_sp
        # ---- device context ----------------------------------------------
        self._create_context()
        self._ctx.upload("U_sp", U_sp)
        self._ctx.upload("U_cv", U_cv)
        self._ctx.upload("W_cv", W_cv)
        self._init_boundaries(U_sp, W_gh)
        if self.potential:
            self.init_potential()
        if self.WB:
            self.init_equilibrium_state()
        self.compute_dt()

    def init_equilibrium_state(self) -> None:
        """The equilibrium of the well-balanced mode, eq_fct(xyz, case)
        (src/sdader_simulator.py:436-481), on the host as in the reference:
        cell means with one ghost element layer, the solution-point and
        conservative values, the flux-point values of every direction with
        each element's left edge set to its left neighbour's right edge, their
        fluxes and, with the FV update, the primitive states and fluxes at the
        subcell faces and the primitives on the extended subcell grid.
        Uploaded to the device (``upload_equilibrium``)."""
        p, n, ndim = self.p, self.p + 1, self.ndim
        W_gh = self.array_sp(ngh=self.Nghe)
        # the quadrature points once for all variables; large grids build
        # them and sum each variable on host thread slabs (bit-identical)
        ncells = int(np.prod(W_gh.shape[1:ndim + 1]))
        workers = min(16, os.cpu_count() or 1) if ncells >= (1 << 15) else 1
        points = quadrature_points_threaded(self.mesh_cv, ndim, workers=workers)
        for var in range(self.nvar):
            W_gh[var] = quadrature_mean(self.mesh_cv, self.eq_fct, ndim, var, points=points, workers=workers)
        del points
        W_sp = self.compute_sp_from_cv(W_gh)
        U_sp = self.compute_conservatives(W_sp)
        eq = {"U_eq_sp": self.crop(U_sp)}
        eq["U_eq_cv"] = self.compute_cv_from_sp(eq["U_eq_sp"])
        for dim in self.dims:
            idim = self.dims[dim]
            vels = np.roll(self.vels, -idim)
            U = self.compute_fp_from_sp(U_sp, dim)
            M_fp = self.crop(U)  # a view: the matching below also changes U
            # elements 1.. along dim take their left edge from the element
            # before (element axis idim+ndim places from the end)
            inner = (slice(None),) * (idim + ndim)
            edge0 = (Ellipsis, 0) + (slice(None),) * idim
            edge1 = (Ellipsis, -1) + (slice(None),) * idim
            M_fp[(Ellipsis, slice(1, None)) + inner][edge0] = M_fp[(Ellipsis, slice(None, -1)) + inner][edge1]
            W = self.compute_primitives(U)
            F = _fluxes(W, vels, self._p_, self.gamma, self.isothermal)
            eq[f"M_eq_fp_{dim}"] = M_fp.copy()
            eq[f"F_eq_fp_{dim}"] = self.crop(F).copy()
            if self.update == "FV":
                last = (Ellipsis, slice(None, -1)) + (slice(None),) * idim
                W_faces = self.integrate_faces(W, dim, ader=False)[last]
                W_faces = self.transpose_to_fv(W_faces)[_crop_fv(p + 1, -p, idim, ndim, p + 1)]
                eq[f"M_eq_faces_{dim}"] = W_faces
                eq[f"F_eq_faces_{dim}"] = _fluxes(W_faces, vels, self._p_, self.gamma, self.isothermal)
        if self.update == "FV":
            ngh = self.Nghc
            M = self.transpose_to_fv(W_gh)
            eq["M_eq_fv"] = M[_crop_fv(n - ngh, -(n - ngh), 0, ndim, n - ngh)] if n > ngh else M
        self.upload_equilibrium(eq)

    def upload_equilibrium(self, eq: dict) -> None:
        """The well-balanced mode's equilibrium arrays (the reference's
        dm.U_eq_sp, U_eq_cv, M_eq_fp_<d>, F_eq_fp_<d>, M_eq_faces_<d>,
        F_eq_faces_<d>, M_eq_fv, in its layouts) to the device; they are
        also kept in ``dm``."""
        for name, arr in eq.items():
            arr = np.ascontiguousarray(arr, dtype=np.float64)
            setattr(self.dm, name, arr)
            self._ctx.upload(name, arr)

    def init_potential(self) -> None:
        """Gradient of the gravity potential phi = init_fct(xyz, -1)
        (src/sdader_simulator.py:425-434): cell means with one ghost element
        layer, the solution-point values, their derivative inside each
        element divided by h, cropped; and its subcell averages.  Host NumPy
        at setup, as in the reference; uploaded to the device."""
        phi_cv = quadrature_mean(self.mesh_cv, self.init_fct, self.ndim, -1)
        phi_sp = self.compute_sp_from_cv(phi_cv[None])
        grad = self.array_sp()[:self.ndim]
        for dim in self.dims:
            idim = self.dims[dim]
            phi_fp = self.compute_fp_from_sp(phi_sp, dim)
            grad[idim] = self.crop(self.compute_sp_from_dfp(phi_fp, dim)) / self.h[dim]
        self.dm.grad_phi_sp = grad
        self.dm.grad_phi_fv = self.transpose_to_fv(self.compute_cv_from_sp(grad))


    # ------------------------------------------------------------------
    # setup
    # ------------------------------------------------------------------
    @staticmethod
    def build_operators(p: int, m: int) -> dict:
        """Constant operators (src/sd_simulator.py:44-52,
        src/sdader_simulator.py:40-44)."""
        x_sp = solution_points(0.0, 1.0, p)
        x_fp = flux_points(0.0, 1.0, p)
        ops = {
            "x_sp": x_sp,
            "x_fp": x_fp,
            "sp_to_fp": lagrange_matrix(x_fp, x_sp),
            "fp_to_sp": lagrange_matrix(x_sp, x_fp),
            "dfp_to_sp": lagrangeprime_matrix(x_sp, x_fp),
            "sp_to_cv": intfromsol_matrix(x_sp, x_fp),
            "fp_to_cv": intfromsol_matrix(x_fp, x_fp),
        }
        ops["cv_to_sp"] = np.linalg.inv(ops["sp_to_cv"])
        x_tp, w_tp = gauss_legendre_quadrature(0.0, 1.0, m + 1)
        ader = ader_matrix(x_tp, w_tp, 1.0)
        invader = np.linalg.inv(ader)
        ops["x_tp"] = x_tp
        ops["w_tp"] = w_tp
        ops["invader"] = np.einsum("p,np->np", w_tp, invader)
        return ops

    def compute_mesh_cv(self) -> np.ndarray:
        return mesh_cv(self.ndim, [self.N[d] for d in self.dims], self.p, [self.lim[d] for d in self.dims],
                       self.Nghe, self.fp["x"])

    def compute_positions(self):
        """Subcell faces, centres and widths with Nghc ghost layers
        (src/sdader_simulator.py:61-92)."""
        ngh = self.Nghc
        self.faces, self.centers, self.h_fp, self.h_cv = {}, {}, {}, {}
        for dim in self.dims:
            idim = self.dims[dim]
            Nd, nd = self.N[dim], self.n[dim]
            fp = subcell_faces(Nd, self.h[dim], self.fp[dim], ngh)
            self.faces[dim] = fp
            cv = 0.5 * (fp[1:] + fp[:-1])
            self.centers[dim] = cv
            self.h_fp[dim] = (fp[1:] - fp[:-1])[self.shape(idim)]
            self.h_cv[dim] = (cv[1:] - cv[:-1])[self.shape(idim)]
            sp = self.lim[dim][0] + (np.arange(Nd)[:, None] + self.sp[dim][None, :]) * self.h[dim]
            setattr(self.dm, f"{dim.upper()}_sp", sp.reshape(Nd, nd))
            setattr(self.dm, f"{dim.upper()}_fp", fp)
            setattr(self.dm, f"{dim.upper()}_cv", cv)

    def _create_context(self):
        cfg = _lib.spd_config()
        cfg.ndim = self.ndim
        for i in range(self.ndim):
            dim = DIMS[i]
            cfg.N[i] = self.N[dim]
            cfg.lim[i][0] = float(self.lim[dim][0])
            cfg.lim[i][1] = float(self.lim[dim][1])
            cfg.BC[i][0] = _lib.BCKIND[self.BC[dim][0]]
            cfg.BC[i][1] = _lib.BCKIND[self.BC[dim][1]]
        cfg.p = self.p
        cfg.m = self.m
        cfg.gamma = self.gamma
        cfg.cfl_coeff = self.cfl_coeff
        cfg.min_c2 = self.min_c2
        cfg.riemann_solver_sd = _lib.RIEMANN[self.riemann_solver_sd_name]
        cfg.riemann_solver_fv = _lib.RIEMANN[self.riemann_solver_fv_name]
        cfg.slope_limiter = _lib.LIMITER[self.slope_limiter_name]
        cfg.update = _lib.UPDATE[self.update]
        cfg.FB = int(bool(self.FB))
        cfg.tolerance = self.tolerance
        cfg.SED = int(bool(self.SED))
        cfg.NAD_delta = int(self.NAD == "delta")
        cfg.PAD = int(bool(self.PAD))
        cfg.blending = int(bool(self.blending))
        cfg.min_rho = self.min_rho
        cfg.max_rho = self.max_rho
        cfg.min_P = self.min_P
        cfg.godunov = int(bool(self.godunov))
        cfg.potential = int(bool(self.potential))
        cfg.isothermal = int(bool(self.isothermal))
        cfg.WB = int(bool(self.WB))
        cfg.viscosity = int(bool(self.viscosity))
        cfg.nu = float(self.nu)
        cfg.beta = float(self.beta)
        faces = [self.faces[DIMS[i]] for i in range(self.ndim)]
        self._ctx = _lib.Context(cfg, self.ops, faces, variant="fma" if self.fma else "ieee")

    def _init_boundaries(self, U_sp, W_gh):
        """Initial boundary arrays: element edge traces of the initial state
        (src/sdader_simulator.py:415-423) and subcell ghost layers of the
        initial condition (src/fv_simulator.py:213-222)."""
        ndim = self.ndim
        T = self.nader
        for dim in self.dims:
            idim = self.dims[dim]
            M_fp = self.compute_fp_from_sp(U_sp, dim)
            first = [slice(None)] * M_fp.ndim
            last = [slice(None)] * M_fp.ndim
            first[-(ndim + idim + 1)] = 0
            first[-(idim + 1)] = 0
            last[-(ndim + idim + 1)] = -1
            last[-(idim + 1)] = -1
            b0 = M_fp[tuple(first)]
            b1 = M_fp[tuple(last)]
            BC = np.stack([np.repeat(b0[:, None], T, axis=1), np.repeat(b1[:, None], T, axis=1)])
            self._ctx.upload(f"BC_fp_{dim}", BC)
        if self.update == "FV":
            ngh = self.Nghc
            n = self.p + 1
            M = self.transpose_to_fv(W_gh)
            if n > 2:
                M = M[(Ellipsis,) + (slice(n - ngh, -(n - ngh)),) * ndim]
            for dim in self.dims:
                idim = self.dims[dim]
                lo = [slice(None)] * M.ndim
                hi = [slice(None)] * M.ndim
                lo[M.ndim - 1 - idim] = slice(None, ngh)
                hi[M.ndim - 1 - idim] = slice(-ngh, None)
                self._ctx.upload(f"BC_fv_{dim}", np.stack([M[tuple(lo)], M[tuple(hi)]]))

    # ------------------------------------------------------------------
    # layouts and host-side helpers (src/sd_simulator.py)
    # ------------------------------------------------------------------
    def array(self, px, py, pz, ngh=0, ader=False) -> np.ndarray:
        shape = [self.nvar, self.nader] if ader else [self.nvar]
        Ns = [self.N[dim] + 2 * ngh for dim in self.dims][::-1]
        pts = [px, py, pz][:self.ndim][::-1]
        return np.ndarray(shape + Ns + pts)

    def array_sp(self, **kwargs):
        return self.array(self.p + 1, self.p + 1, self.p + 1, **kwargs)

    def array_fp(self, dims="xyz", **kwargs):
        """Flux-point array shape (src/sd_simulator.py:150-156)."""
        p = self.p
        return self.array(p + 1 + ("x" in dims), p + 1 + ("y" in dims), p + 1 + ("z" in dims), **kwargs)

    def array_RS(self, dim="x", ader=False) -> np.ndarray:
        """Riemann-problem array shape (src/sd_simulator.py:158-166)."""
        shape = [self.nvar, self.nader] if ader else [self.nvar]
        shape += [self.N[d2] + (d2 == dim) for d2 in self.dims][::-1]
        shape += [self.p + 1] * (self.ndim - 1)
        return np.ndarray(shape)

    def array_BC(self, dim="x", ader=False) -> np.ndarray:
        """Domain-boundary array shape (src/sd_simulator.py:168-182)."""
        shape = [2, self.nvar, self.nader] if ader else [2, self.nvar]
        if self.Z and dim in ("x", "y"):
            shape += [self.N["z"]]
        if self.Y and dim in ("x", "z"):
            shape += [self.N["y"]]
        if dim in ("y", "z"):
            shape += [self.N["x"]]
        shape += [self.p + 1] * (self.ndim - 1)
        return np.ndarray(shape)

    def integrate_faces(self, M_fp, dim, ader=True):
        """Subcell averages across the directions other than ``dim``
        (src/sd_simulator.py:208-212)."""
        for other in self.dims:
            if other != dim:
                M_fp = transform_axis(M_fp, self.ops["sp_to_cv"], self.dims[other], self.ndim, ader=ader)
        return M_fp

    def compute_sp_from_dfp_x(self, ader=True):
        """src/sd_simulator.py:199-200 on ``dm.F_ader_fp_x``."""
        return self.compute_sp_from_dfp(self.dm.F_ader_fp_x, "x", ader=ader) / self.dx

    def compute_sp_from_dfp_y(self, ader=True):
        return self.compute_sp_from_dfp(self.dm.F_ader_fp_y, "y", ader=ader) / self.dy

    def compute_sp_from_dfp_z(self, ader=True):
        return self.compute_sp_from_dfp(self.dm.F_ader_fp_z, "z", ader=ader) / self.dz

    def _F_ader_fp(self, d):
        """``dm.F_ader_fp_<d>`` after a step with the FV update: the last
        Picard iteration's flux-point fluxes averaged across the other
        directions (what the reference's array holds after
        switch_to_finite_volume, src/sdader_simulator.py:297-298), in its
        layout (V, T, [Nz,] [Ny,] Nx, [nz,] [ny,] nx) with p+2 points along
        d.  The SD update keeps no flux-point array on the device."""
        if d not in self.dims:
            raise AttributeError(f"F_ader_fp_{d}")
        if self.update != "FV":
            raise AttributeError(f"F_ader_fp_{d} is kept on the device only with update='FV'")
        idim = self.dims[d]
        n, T, V, nd = self.p + 1, self.nader, self.nvar, self.ndim
        X = [self.N[DIMS[i]] * n for i in range(nd)]
        FX = [X[i] + (1 if i == idim else 0) for i in range(nd)]
        raw = self._ctx.download(f"F_faces_{d}", (T, V, int(np.prod(FX))))
        # face index of (cell c_i, point k_i): coordinate c_i*n + k_i along
        # each direction i, faces x-fastest; reference axes are
        # (cells z, y, x, points z, y, x) for the directions present
        fid = np.zeros([1] * (2 * nd), dtype=np.int64)
        stride = 1
        for i in range(nd):
            npts = n + 1 if i == idim else n
            coord = np.arange(self.N[DIMS[i]])[:, None] * n + np.arange(npts)[None, :]
            shp = [1] * (2 * nd)
            shp[nd - 1 - i] = self.N[DIMS[i]]
            shp[2 * nd - 1 - i] = npts
            # place the (cell, point) grid on axes (nd-1-i, 2nd-1-i)
            fid = fid + np.moveaxis(coord.reshape(coord.shape + (1,) * (2 * nd - 2)), [0, 1],
                                    [nd - 1 - i, 2 * nd - 1 - i]).reshape(shp) * stride
            stride *= FX[i]
        return np.ascontiguousarray(raw[:, :, fid].transpose((1, 0) + tuple(range(2, 2 + 2 * nd))))

    def transpose_to_fv(self, M):
        if self.ndim == 1:
            return M.reshape(M.shape[0], M.shape[1] * M.shape[2])
        if self.ndim == 2:
            return np.transpose(M, (0, 1, 3, 2, 4)).reshape(M.shape[0], M.shape[1] * M.shape[3],
                                                            M.shape[2] * M.shape[4])
        return np.transpose(M, (0, 1, 4, 2, 5, 3, 6)).reshape(M.shape[0], M.shape[1] * M.shape[4],
                                                              M.shape[2] * M.shape[5], M.shape[3] * M.shape[6])

    def transpose_to_sd(self, M):
        shape = []
        for dim in self.dims:
            shape += [self.n[dim], self.N[dim]]
        shape = [M.shape[0]] + shape[::-1]
        if self.ndim == 1:
            return M.reshape(shape)
        if self.ndim == 2:
            return np.transpose(M.reshape(shape), (0, 1, 3, 2, 4))
        return np.transpose(M.reshape(shape), (0, 1, 3, 5, 2, 4, 6))

    def compute_sp_from_cv(self, M_cv) -> np.ndarray:
        return transform_full(M_cv, self.ops["cv_to_sp"], self.ndim)

    def compute_cv_from_sp(self, M_sp) -> np.ndarray:
        return transform_full(M_sp, self.ops["sp_to_cv"], self.ndim)

    def compute_fp_from_sp(self, M_sp, dim, **kwargs) -> np.ndarray:
        return transform_axis(M_sp, self.ops["sp_to_fp"], self.dims[dim], self.ndim, **kwargs)

    def compute_sp_from_fp(self, M_fp, dim, **kwargs) -> np.ndarray:
        return transform_axis(M_fp, self.ops["fp_to_sp"], self.dims[dim], self.ndim, **kwargs)

    def compute_sp_from_dfp(self, M_fp, dim, **kwargs) -> np.ndarray:
        return transform_axis(M_fp, self.ops["dfp_to_sp"], self.dims[dim], self.ndim, **kwargs)

    def regular_mesh(self, W):
        """Interpolate SD-layout values to equispaced points for plotting
        (src/sd_simulator.py:92-102)."""
        p = self.p
        if p <= 1:
            return W
        x = np.arange(p + 2) / (p + 1)
        x = .5 * (x[1:] + x[:-1])
        return transform_full(W, lagrange_matrix(x, solution_points(0.0, 1.0, p)), self.ndim)

    # ------------------------------------------------------------------
    # device state
    # ------------------------------------------------------------------
    def _shape_of(self, name):
        nd = self.ndim
        Ns = tuple(self.N[DIMS[i]] for i in range(nd))[::-1]
        n = self.p + 1
        X = [self.N[DIMS[i]] * n for i in range(nd)]
        if name in ("U_sp", "U_cv", "W_cv"):
            return (self.nvar,) + Ns + (n,) * nd
        if name == "troubles":
            return (1,) + tuple(X[::-1])
        if name == "theta":
            return (1,) + tuple(x + 2 * self.Nghc for x in X[::-1])
        if name.startswith("affected_faces_"):
            d = DIMS.index(name[-1])
            ext = [x + (1 if i == d else 0) for i, x in enumerate(X)]
            return (1,) + tuple(ext[::-1])
        raise KeyError(name)

    def _download(self, name):
        if name.startswith("affected_faces_") and DIMS.index(name[-1]) >= self.ndim:
            raise AttributeError(name)
        if name in ("troubles", "theta") or name.startswith("affected_faces_"):
            if not (self.update == "FV" and self.FB):
                raise AttributeError(f"{name} exists only with update='FV' and FB=True")
        return self._ctx.download(name, self._shape_of(name))

    # ------------------------------------------------------------------
    # time stepping (src/sdader_simulator.py:361-413, src/sd_simulator.py:214-227)
    # ------------------------------------------------------------------
    def compute_dt(self) -> None:
        self._ctx.compute_dt()

    def perform_update(self) -> bool:
        self.n_step += 1
        self.time = self._ctx.perform_update(self.time)
        return True

    def init_sim(self):
        self.execution_time = -timer()

    def end_sim(self):
        self._ctx.synchronize()
        self.execution_time += timer()
        self._ctx.end_sim()
        if self.rank == 0:
            print(f"t={self.time}, steps taken {self.n_step}, time taken {self.execution_time}")

    @staticmethod
    def _warn_nonfinite(nonfinite: bool) -> None:
        if nonfinite:
            warnings.warn("non-finite dt: the state holds NaN or inf (the steps ran as in the reference)",
                          RuntimeWarning, stacklevel=3)

    def perform_iterations(self, n_step: int) -> None:
        self.init_sim()
        self.time, done, nonfinite = self._ctx.step(n_step, 0.0, 0, self.time)
        self.n_step += done
        self.end_sim()
        self._warn_nonfinite(nonfinite)

    def perform_time_evolution(self, t_end: float, nsteps=0) -> None:
        self.init_sim()
        self.time, done, nonfinite = self._ctx.step(0, t_end, 1, self.time)
        self.n_step += done
        if self.time < t_end:
            print(f"dt={self.dm.dt}")
        self.end_sim()
        self._warn_nonfinite(nonfinite)

    # ------------------------------------------------------------------
    # state snapshots (no counterpart in the reference, which has no
    # save/load): the device state, time, step count and dt in one .npz
    # ------------------------------------------------------------------
    def _snapshot_config(self) -> dict:
        return dict(ndim=self.ndim, N=[self.N[d] for d in self.dims], p=self.p, m=self.m, update=self.update,
                    FB=bool(self.FB), riemann_solver_sd=self.riemann_solver_sd_name,
                    riemann_solver_fv=self.riemann_solver_fv_name, slope_limiter=self.slope_limiter_name,
                    BC=[list(self.BC[d]) for d in self.dims], gamma=self.gamma, cfl_coeff=self.cfl_coeff,
                    lims=[list(self.lim[d]) for d in self.dims], viscosity=bool(self.viscosity), nu=self.nu,
                    beta=self.beta, potential=bool(self.potential), isothermal=bool(self.isothermal),
                    WB=bool(self.WB))

    def save_state(self, path) -> None:
        """Write U_sp, U_cv, W_cv, the FV boundary buffers, time, n_step, dt
        and the configuration to ``path`` (.npz)."""
        import json
        arrays = {name: self._download(name) for name in ("U_sp", "U_cv", "W_cv")}
        if self.update == "FV":
            for d in self.dims:
                idim = self.dims[d]
                ext = [self.N[DIMS[i]] * (self.p + 1) + 2 * self.Nghc for i in range(self.ndim)]
                ext[idim] = self.Nghc
                arrays[f"BC_fv_{d}"] = self._ctx.download(f"BC_fv_{d}", (2, self.nvar) + tuple(ext[::-1]))
        np.savez(path, time=np.float64(self.time), n_step=np.int64(self.n_step), dt=np.float64(self._ctx.get_dt()),
                 config=json.dumps(self._snapshot_config()), **arrays)

    def restore_state(self, path) -> None:
        """Load a snapshot written by ``save_state`` of a simulator built with
        the same configuration; the run then continues bit for bit."""
        import json
        z = np.load(path)
        cfg = json.loads(str(z["config"]))
        if cfg != json.loads(json.dumps(self._snapshot_config())):
            raise ValueError(f"snapshot configuration differs: {cfg}")
        for name in ("U_sp", "U_cv", "W_cv"):
            self._ctx.upload(name, z[name])
        if self.update == "FV":
            for d in self.dims:
                self._ctx.upload(f"BC_fv_{d}", z[f"BC_fv_{d}"])
        self.time = float(z["time"])
        self.n_step = int(z["n_step"])
        self._ctx.set_dt(float(z["dt"]))

    def close(self):
        if self._ctx is not None:
            self._ctx.close()
            self._ctx = None


class SDADER_Simulator(SD_Simulator, FV_Simulator):
    """SD-ADER simulator for the compressible Euler equations (GPU step).

    Positional and keyword arguments follow the reference's constructor
    chain SDADER_Simulator -> SD_Simulator -> FV_Simulator -> Simulator
    (src/sdader_simulator.py:14-59).

    Two keywords have no counterpart in the reference: ``operators`` (the
    constant operator matrices, when the caller has them already) and
    ``fma``: True runs the step from the library built with fused
    multiply-adds (one FP64 instruction and one rounding per a*b+c instead
    of two), which is faster but no longer bit-identical to the reference.
    """

    def __init__(self,
                 FB: bool = False,
                 tolerance: float = 1e-5,
                 SED: bool = True,
                 NAD: str = "",
                 PAD: bool = True,
                 blending: bool = True,
                 min_rho: float = 1e-10,
                 max_rho: float = 1e10,
                 min_P: float = 1e-10,
                 godunov: bool = False,
                 *args,
                 operators: dict | None = None,
                 fma: bool = False,
                 **kwargs):
        self._ctx = None
        # the SDADER options are set before the chain below runs, because
        # SD_Simulator creates the device context with all of them
        self.FB = FB
        self.tolerance = tolerance
        self.SED = SED
        self.NAD = NAD
        self.PAD = PAD
        self.blending = blending
        self.min_rho = min_rho
        self.max_rho = max_rho
        self.min_P = min_P
        self.godunov = godunov
        self._operators = operators
        self.fma = bool(fma)
        super().__init__(*args, **kwargs)

    def array_FV(self, n, nvar, dim=None, ngh=0) -> np.ndarray:
        """src/sdader_simulator.py:273-278 (n subcells per cell and
        direction)."""
        N = [self.N[d2] * n + (dim == d2) + 2 * ngh for d2 in self.dims]
        return np.ndarray([nvar] + N[::-1])

    def array_FV_BC(self, dim="x") -> np.ndarray:
        """src/sdader_simulator.py:280-286."""
        ngh = self.Nghc
        N = [self.N[d2] * self.n[d2] + 2 * ngh if dim != d2 else ngh for d2 in self.dims]
        return np.ndarray([2, self.nvar] + N[::-1])

