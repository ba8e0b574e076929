"""Generate the golden fixtures in this directory by running the reference.

Run once in a container where the reference's sources are present:

    python tests/golden/make_golden.py /path/to/reference [--only name,name] [--long]

It imports the reference's NumPy implementation (``src/`` of jpalafou/spd,
CuPy absent so the FP64 NumPy path runs), builds each case below, records
the constant operators and the initial state, advances the listed number of
steps with ``compute_dt`` + ``perform_update`` (the body of
``perform_iterations``) and records the state after every case.  The
fixtures are .npz files; ``case.json`` inside each describes the run.

``--long`` makes the long-horizon fixtures in ``long/`` instead: 100 steps
(or a run to t_end with the clip and stop of ``perform_time_evolution``),
with the dt of every step and, with limiting, a CRC-32 and a count of the
trouble mask after every step; the t_end vortex case also stores the L1
density error against the exact (translated) vortex, computed with the
reference's own quadrature.
"""
from __future__ import annotations

import json
import os
import sys
import warnings

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
from spd_gb300 import initial_conditions as ics  # noqa: E402

# name -> (constructor kwargs, initial condition spec, steps)
CASES = {
    "vortex32_p3_fvfb_llf": (dict(p=3, N=(32, 32), xlim=(0, 10), ylim=(0, 10), update="FV", FB=True,
                                  riemann_solver_sd="llf", riemann_solver_fv="llf", cfl_coeff=0.8,
                                  BC=(("periodic", "periodic"),) * 2), ("vortex", {}), 1),
    "quadrant16_p3_fvfb_hllc_gradfree": (dict(p=3, N=(16, 16), update="FV", FB=True, riemann_solver_sd="hllc",
                                              riemann_solver_fv="hllc", BC=(("gradfree", "gradfree"),) * 2),
                                         ("four_quadrant", {}), 5),
    "sedov6_p2_fvfb_hllc_reflective": (dict(p=2, N=(6, 6, 6), update="FV", FB=True, riemann_solver_sd="hllc",
                                            riemann_solver_fv="hllc", BC=(("reflective", "reflective"),) * 3),
                                       ("sedov", {"N": 6}), 3),
    "sod32_p3_fvfb_hllc_gradfree": (dict(p=3, N=(32,), update="FV", FB=True, riemann_solver_sd="hllc",
                                         riemann_solver_fv="hllc", BC=(("gradfree", "gradfree"),)),
                                    ("sod", {}), 10),
    "step8_p1_sd_llf_periodic": (dict(p=1, N=(8, 8), update="SD", FB=False, riemann_solver_sd="llf",
                                      BC=(("periodic", "periodic"),) * 2), ("step_function", {}), 10),
    "sine4_p3_sd_hllc_periodic_3d": (dict(p=3, N=(4, 4, 4), update="SD", riemann_solver_sd="hllc",
                                          BC=(("periodic", "periodic"),) * 3), ("sine_wave", {}), 2),
    "kh16_p3_fvfb_hllc_moncen": (dict(p=3, N=(16, 16), update="FV", FB=True, riemann_solver_sd="hllc",
                                      riemann_solver_fv="hllc", slope_limiter="moncen",
                                      BC=(("periodic", "periodic"),) * 2), ("kelvin_helmholtz", {"N": 16}), 3),
    "quadrant8_p2_godunov_delta_lhllc_reflective": (dict(p=2, N=(8, 8), update="FV", FB=True, godunov=True,
                                                         NAD="delta", riemann_solver_sd="lhllc",
                                                         riemann_solver_fv="lhllc",
                                                         BC=(("reflective", "reflective"),) * 2),
                                                    ("four_quadrant", {}), 3),
    "quadrant12_p3_fv_noblend_nosed": (dict(p=3, N=(12, 12), update="FV", FB=True, blending=False, SED=False,
                                            riemann_solver_sd="hllc", riemann_solver_fv="llf",
                                            BC=(("gradfree", "reflective"), ("periodic", "periodic"))),
                                       ("four_quadrant", {}), 3),
    # degree 4, time orders m != p, the fixed-state boundaries (ic,
    # pressure), another gamma and CFL, PAD off, p=1 in 3D
    "quadrant8_p4_fvfb_hllc_gradfree": (dict(p=4, N=(8, 8), update="FV", FB=True, riemann_solver_sd="hllc",
                                             riemann_solver_fv="hllc", BC=(("gradfree", "gradfree"),) * 2),
                                        ("four_quadrant", {}), 3),
    "quadrant8_p3_m1_fvfb_ic_pressure": (dict(p=3, m=1, N=(8, 8), update="FV", FB=True, riemann_solver_sd="hllc",
                                              riemann_solver_fv="hllc", BC=(("ic", "ic"), ("pressure", "pressure"))),
                                         ("four_quadrant", {}), 3),
    "sine24_p4_m2_sd_lhllc_ic": (dict(p=4, m=2, N=(24,), update="SD", riemann_solver_sd="lhllc",
                                      BC=(("ic", "gradfree"),)), ("sine_wave", {}), 5),
    "vortex16_p2_m4_fv_llf_gamma53": (dict(p=2, m=4, N=(16, 16), xlim=(0, 10), ylim=(0, 10), update="FV", FB=False,
                                           riemann_solver_sd="llf", gamma=5.0 / 3.0, cfl_coeff=0.5,
                                           BC=(("periodic", "periodic"),) * 2), ("vortex", {}), 3),
    "kh8_p3_fvfb_nopad_moncen_mixed": (dict(p=3, N=(8, 8), update="FV", FB=True, PAD=False,
                                            slope_limiter="moncen", riemann_solver_sd="lhllc",
                                            riemann_solver_fv="hllc",
                                            BC=(("reflective", "pressure"), ("ic", "gradfree"))),
                                       ("kelvin_helmholtz", {"N": 8}), 3),
    "quadrant8_p2_fv_nofb_hllc_eq": (dict(p=2, N=(8, 8), update="FV", FB=False, riemann_solver_sd="hllc",
                                          BC=(("eq", "gradfree"), ("periodic", "eq"))), ("four_quadrant", {}), 3),
    "sine6_p1_fvfb_llf_3d": (dict(p=1, N=(6, 6, 6), update="FV", FB=True, riemann_solver_sd="llf",
                                  riemann_solver_fv="llf", BC=(("periodic", "periodic"),) * 3), ("sine_wave", {}), 3),
    # viscosity (src/sdader_simulator.py:245-268): SD update and the FV
    # update without limiting (with FB=True the reference's viscous fallback
    # fluxes raise AttributeError, src/muscl.py:253, src/muscl.py:97)
    "visc_sine8_p2_sd_llf_periodic_dtclamp": (dict(p=2, N=(8, 8), update="SD", riemann_solver_sd="llf",
                                                   viscosity=True, nu=0.05,
                                                   BC=(("periodic", "periodic"),) * 2),
                                              ("sine_wave", {}), 6),
    "visc_kh16_p3_fv_hllc_periodic": (dict(p=3, N=(16, 16), update="FV", FB=False, riemann_solver_sd="hllc",
                                           viscosity=True, nu=1e-3, BC=(("periodic", "periodic"),) * 2),
                                      ("kelvin_helmholtz", {"N": 16}), 4),
    "visc_quadrant8_p2_sd_hllc_mixed_bc": (dict(p=2, N=(8, 8), update="SD", riemann_solver_sd="hllc",
                                                viscosity=True, nu=2e-3, beta=0.5,
                                                BC=(("reflective", "gradfree"), ("ic", "pressure"))),
                                           ("four_quadrant", {}), 4),
    "visc_sedov4_p2_fv_llf_reflective_3d": (dict(p=2, N=(4, 4, 4), update="FV", riemann_solver_sd="llf",
                                                 viscosity=True, nu=1e-3,
                                                 BC=(("reflective", "reflective"),) * 3),
                                            ("sedov", {"N": 4}), 3),
    "visc_sine16_p3_sd_llf_eq": (dict(p=3, N=(16,), update="SD", riemann_solver_sd="llf", viscosity=True, nu=1e-3,
                                      BC=(("eq", "eq"),)), ("sine_wave", {}), 5),
    # gravity potential (src/sdader_simulator.py:425-434, src/simulator.py:197-203)
    "pot_column8_p2_sd_hllc_reflective": (dict(p=2, N=(8, 8), update="SD", riemann_solver_sd="hllc", potential=True,
                                               BC=(("periodic", "periodic"), ("reflective", "reflective"))),
                                          ("gravity_column", {}), 5),
    "pot_column8_p3_fvfb_hllc_gradfree": (dict(p=3, N=(8, 8), update="FV", FB=True, riemann_solver_sd="hllc",
                                               riemann_solver_fv="hllc", potential=True,
                                               BC=(("periodic", "periodic"), ("gradfree", "gradfree"))),
                                          ("gravity_column", {"g": 2.0, "amp": 0.5, "step": True}), 4),
    "pot_column4_p2_fv_llf_3d": (dict(p=2, N=(4, 3, 5), update="FV", riemann_solver_sd="llf", potential=True,
                                      BC=(("periodic", "periodic"), ("periodic", "periodic"),
                                          ("reflective", "reflective"))),
                                 ("gravity_column", {"g": 1.5}), 3),
    "pot_visc_column16_p3_sd_llf_1d": (dict(p=3, N=(16,), update="SD", riemann_solver_sd="llf", potential=True,
                                            viscosity=True, nu=1e-3, BC=(("reflective", "reflective"),)),
                                       ("gravity_column", {}), 4),
    # isothermal system (src/hydro.py:84,123,169, src/riemann_solver.py:142,210)
    "iso_quadrant8_p2_fvfb_hllc_gradfree": (dict(p=2, N=(8, 8), update="FV", FB=True, riemann_solver_sd="hllc",
                                                 riemann_solver_fv="hllc", isothermal=True,
                                                 BC=(("gradfree", "gradfree"),) * 2),
                                            ("four_quadrant", {}), 4),
    "iso_sine16_p3_sd_llf_periodic": (dict(p=3, N=(16,), update="SD", riemann_solver_sd="llf", isothermal=True,
                                           BC=(("periodic", "periodic"),)), ("sine_wave", {}), 5),
    "iso_pot_column8_p2_fv_lhllc": (dict(p=2, N=(8, 8), update="FV", FB=True, riemann_solver_sd="lhllc",
                                         riemann_solver_fv="llf", isothermal=True, potential=True,
                                         BC=(("periodic", "periodic"), ("reflective", "reflective"))),
                                    ("gravity_column", {"amp": 0.3, "step": True}), 3),
    # well-balanced mode (src/sdader_simulator.py:436-481 and its uses):
    # ``eq_ic`` is the equilibrium state's initial condition (eq_fct)
    "wb_column8_p2_fvfb_hllc_eq": (dict(p=2, N=(8, 8), update="FV", FB=True, riemann_solver_sd="hllc",
                                        riemann_solver_fv="hllc", WB=True, potential=True,
                                        eq_ic=["gravity_column", {"amp": 0.0}],
                                        BC=(("periodic", "periodic"), ("eq", "eq"))),
                                   ("gravity_column", {"amp": 0.05, "step": True}), 5),
    "wb_column8_p3_sd_hllc_reflective": (dict(p=3, N=(8, 8), update="SD", riemann_solver_sd="hllc", WB=True,
                                              potential=True, eq_ic=["gravity_column", {"amp": 0.0}],
                                              BC=(("periodic", "periodic"), ("reflective", "reflective"))),
                                         ("gravity_column", {"amp": 0.05}), 5),
    "wb_column8_p2_fv_llf_eq": (dict(p=2, N=(8, 8), update="FV", riemann_solver_sd="llf", WB=True,
                                     potential=True, eq_ic=["gravity_column", {"amp": 0.0}],
                                     BC=(("periodic", "periodic"), ("eq", "eq"))),
                                ("gravity_column", {"amp": 0.05}), 4),
    "wb_sine8_p3_fvfb_moncen_periodic": (dict(p=3, N=(8, 8), update="FV", FB=True, riemann_solver_sd="hllc",
                                              riemann_solver_fv="llf", slope_limiter="moncen", WB=True,
                                              eq_ic=["sine_wave", {}], BC=(("periodic", "periodic"),) * 2),
                                         ("step_function", {}), 4),
    "wb_column4_p2_fvfb_hllc_3d": (dict(p=2, N=(4, 3, 4), update="FV", FB=True, riemann_solver_sd="hllc",
                                        riemann_solver_fv="hllc", WB=True, potential=True,
                                        eq_ic=["gravity_column", {"amp": 0.0, "g": 1.5}],
                                        BC=(("periodic", "periodic"), ("periodic", "periodic"), ("eq", "eq"))),
                                   ("gravity_column", {"amp": 0.05, "g": 1.5, "step": True}), 3),
    "wb_visc_column8_p2_sd_llf": (dict(p=2, N=(8, 8), update="SD", riemann_solver_sd="llf", WB=True,
                                       potential=True, viscosity=True, nu=1e-3,
                                       eq_ic=["gravity_column", {"amp": 0.0}],
                                       BC=(("periodic", "periodic"), ("eq", "eq"))),
                                  ("gravity_column", {"amp": 0.05}), 3),
    "wb_iso_column8_p2_fvfb_hllc": (dict(p=2, N=(8, 8), update="FV", FB=True, riemann_solver_sd="hllc",
                                         riemann_solver_fv="hllc", WB=True, potential=True, isothermal=True,
                                         eq_ic=["gravity_column", {"amp": 0.0}],
                                         BC=(("periodic", "periodic"), ("reflective", "reflective"))),
                                    ("gravity_column", {"amp": 0.05, "step": True}), 3),
}


# long-horizon cases: name -> (constructor kwargs, initial condition spec,
# {"steps": n} or {"t_end": t})
LONG_CASES = {
    "vortex32_p3_fvfb_llf_100steps": (CASES["vortex32_p3_fvfb_llf"][0], ("vortex", {}), {"steps": 100}),
    "vortex32_p3_fvfb_llf_t1": (CASES["vortex32_p3_fvfb_llf"][0], ("vortex", {}), {"t_end": 1.0}),
    "quadrant32_p3_fvfb_hllc_gradfree_100steps": (dict(p=3, N=(32, 32), update="FV", FB=True,
                                                       riemann_solver_sd="hllc", riemann_solver_fv="hllc",
                                                       BC=(("gradfree", "gradfree"),) * 2),
                                                  ("four_quadrant", {}), {"steps": 100}),
    # at 8^3 the reference's state takes negative densities from step ~20
    # and becomes NaN at step 63: 60 steps pin the near-vacuum path
    "sedov8_p2_fvfb_hllc_reflective_60steps": (dict(p=2, N=(8, 8, 8), update="FV", FB=True,
                                                    riemann_solver_sd="hllc", riemann_solver_fv="hllc",
                                                    BC=(("reflective", "reflective"),) * 3),
                                               ("sedov", {"N": 8}), {"steps": 60}),
    # the final state of this one is stored as CRC-32 digests of its bytes
    # (with its sum and largest magnitude), which keeps the fixture small
    "sedov16_p2_fvfb_hllc_reflective_100steps": (dict(p=2, N=(16, 16, 16), update="FV", FB=True,
                                                      riemann_solver_sd="hllc", riemann_solver_fv="hllc",
                                                      BC=(("reflective", "reflective"),) * 3),
                                                 ("sedov", {"N": 16}), {"steps": 100, "digest_state": True}),
    "kh32_p3_fvfb_hllc_moncen_100steps": (dict(p=3, N=(32, 32), update="FV", FB=True, riemann_solver_sd="hllc",
                                               riemann_solver_fv="hllc", slope_limiter="moncen",
                                               BC=(("periodic", "periodic"),) * 2),
                                          ("kelvin_helmholtz", {"N": 32}), {"steps": 100}),
    "sod64_p2_fvfb_llf_gradfree_t02": (dict(p=2, N=(64,), update="FV", FB=True, riemann_solver_sd="llf",
                                            riemann_solver_fv="llf", BC=(("gradfree", "gradfree"),)),
                                       ("sod", {}), {"t_end": 0.2}),
    "visc_kh32_p3_sd_hllc_periodic_100steps": (dict(p=3, N=(32, 32), update="SD", riemann_solver_sd="hllc",
                                                    viscosity=True, nu=1e-3, BC=(("periodic", "periodic"),) * 2),
                                               ("kelvin_helmholtz", {"N": 32}), {"steps": 100}),
    "wb_column16_p3_fvfb_hllc_eq_100steps": (dict(p=3, N=(16, 16), update="FV", FB=True, riemann_solver_sd="hllc",
                                                  riemann_solver_fv="hllc", WB=True, potential=True,
                                                  eq_ic=["gravity_column", {"amp": 0.0}],
                                                  BC=(("periodic", "periodic"), ("eq", "eq"))),
                                             ("gravity_column", {"amp": 0.05, "step": True}), {"steps": 100}),
    "step16_p3_sd_hllc_periodic_100steps": (dict(p=3, N=(16, 16), update="SD", riemann_solver_sd="hllc",
                                                 BC=(("periodic", "periodic"),) * 2),
                                            ("step_function", {}), {"steps": 100}),
}


def ref_kwargs(kw):
    """Constructor keywords of a case: ``eq_ic`` becomes the eq_fct callback."""
    kw = dict(kw)
    if "eq_ic" in kw:
        kw["eq_fct"] = make_ic(tuple(kw.pop("eq_ic")))
    return kw


def eq_arrays(s):
    """The equilibrium arrays of the well-balanced mode
    (src/sdader_simulator.py:436-481), when it is on."""
    out = {}
    if not s.WB:
        return out
    out["U_eq_sp"] = s.dm.U_eq_sp.copy()
    out["U_eq_cv"] = s.dm.U_eq_cv.copy()
    for d in s.dims:
        out[f"M_eq_fp_{d}"] = getattr(s.dm, f"M_eq_fp_{d}").copy()
        out[f"F_eq_fp_{d}"] = getattr(s.dm, f"F_eq_fp_{d}").copy()
        if s.update == "FV":
            out[f"M_eq_faces_{d}"] = getattr(s.dm, f"M_eq_faces_{d}").copy()
            out[f"F_eq_faces_{d}"] = getattr(s.dm, f"F_eq_faces_{d}").copy()
    if s.update == "FV":
        out["M_eq_fv"] = s.dm.M_eq_fv.copy()
    return out


def make_ic(spec):
    name, kw = spec
    if name == "vortex":
        return ics.isentropic_vortex()
    if name in ("sedov", "kelvin_helmholtz", "gravity_column"):
        return getattr(ics, name)(**kw)
    return getattr(ics, name)


def main(ref_root, only=None, long=False):
    sys.path.insert(0, os.path.join(ref_root, "src"))
    warnings.simplefilter("ignore")
    from sdader_simulator import SDADER_Simulator  # the reference
    import polynomials as rpoly
    if long:
        return main_long(SDADER_Simulator, rpoly, only)

    # setup operators for p = 1..4 (host-side pin)
    ops = {}
    for p in range(1, 5):
        x_sp = rpoly.solution_points(0.0, 1.0, p)
        x_fp = rpoly.flux_points(0.0, 1.0, p)
        ops[f"p{p}_x_sp"] = x_sp
        ops[f"p{p}_x_fp"] = x_fp
        ops[f"p{p}_sp_to_fp"] = rpoly.lagrange_matrix(x_fp, x_sp)
        ops[f"p{p}_dfp_to_sp"] = rpoly.lagrangeprime_matrix(x_sp, x_fp)
        ops[f"p{p}_sp_to_cv"] = rpoly.intfromsol_matrix(x_sp, x_fp)
        x_tp, w_tp = rpoly.gauss_legendre_quadrature(0.0, 1.0, p + 1)
        ops[f"p{p}_x_tp"] = x_tp
        ops[f"p{p}_w_tp"] = w_tp
        ops[f"p{p}_ader"] = rpoly.ader_matrix(x_tp, w_tp, 1.0)
    np.savez_compressed(os.path.join(HERE, "operators.npz"), **ops)

    for name, (kw, icspec, steps) in CASES.items():
        if only and name not in only:
            continue
        init = make_ic(icspec)
        s = SDADER_Simulator(init_fct=init, use_cupy=False, verbose=False, **ref_kwargs(kw))
        out = {
            "sp_to_fp": s.dm.sp_to_fp, "fp_to_sp": s.dm.fp_to_sp, "dfp_to_sp": s.dm.dfp_to_sp,
            "sp_to_cv": s.dm.sp_to_cv, "fp_to_cv": s.dm.fp_to_cv, "cv_to_sp": s.dm.cv_to_sp,
            "x_tp": s.dm.x_tp, "w_tp": s.dm.w_tp, "invader": s.dm.invader, "x_sp": s.x_sp, "x_fp": s.x_fp,
            "init_U_sp": s.dm.U_sp.copy(), "init_U_cv": s.dm.U_cv.copy(), "init_W_cv": s.dm.W_cv.copy(),
        }
        for d in s.dims:
            out[f"init_BC_fp_{d}"] = getattr(s.dm, f"BC_fp_{d}").copy()
            if s.update == "FV":
                out[f"init_BC_fv_{d}"] = getattr(s.dm, f"BC_fv_{d}").copy()
        if s.potential:
            out["grad_phi_sp"] = s.dm.grad_phi_sp.copy()
            out["grad_phi_fv"] = s.dm.grad_phi_fv.copy()
        out.update(eq_arrays(s))
        s.init_sim()
        dts = []
        for _ in range(steps):
            s.compute_dt()
            dts.append(float(s.dm.dt))
            s.perform_update()
        out["dts"] = np.array(dts)
        out["time"] = np.array(s.time)
        if not np.abs(s.dm.U_sp).max() < 1e3:
            # a run that blew up pins only arithmetic, not a solution
            raise RuntimeError(f"{name}: the reference's state left the physical range "
                               f"(max |U_sp| = {np.abs(s.dm.U_sp).max():.3g}); choose a stable case")
        out["U_sp"] = s.dm.U_sp.copy()
        out["U_cv"] = s.dm.U_cv.copy()
        out["W_cv"] = s.dm.W_cv.copy()
        if s.update == "FV" and s.FB:
            out["troubles"] = s.dm.troubles.copy()
            out["theta"] = s.dm.theta.copy()
            for d in s.dims:
                out[f"affected_faces_{d}"] = getattr(s.dm, f"affected_faces_{d}").copy()
        meta = dict(kwargs={k: (list(map(list, v)) if k == "BC" else (list(v) if isinstance(v, tuple) else v))
                            for k, v in kw.items()},
                    ic=list(icspec), steps=steps)
        out["case_json"] = np.array(json.dumps(meta))
        np.savez_compressed(os.path.join(HERE, f"{name}.npz"), **out)
        print(name, "steps", steps, "troubles", float(s.dm.troubles.sum()) if "troubles" in out else "-",
              os.path.getsize(os.path.join(HERE, f"{name}.npz")) // 1024, "KB", flush=True)


def _trouble_digest(s):
    import zlib
    t = np.ascontiguousarray(s.dm.troubles)
    return zlib.crc32(t.tobytes()), float(t.sum())


def main_long(SDADER_Simulator, rpoly, only):
    out_dir = os.path.join(HERE, "long")
    os.makedirs(out_dir, exist_ok=True)
    for name, (kw, icspec, run) in LONG_CASES.items():
        if only and name not in only:
            continue
        init = make_ic(icspec)
        s = SDADER_Simulator(init_fct=init, use_cupy=False, verbose=False, **ref_kwargs(kw))
        out = {
            "sp_to_fp": s.dm.sp_to_fp, "fp_to_sp": s.dm.fp_to_sp, "dfp_to_sp": s.dm.dfp_to_sp,
            "sp_to_cv": s.dm.sp_to_cv, "fp_to_cv": s.dm.fp_to_cv, "cv_to_sp": s.dm.cv_to_sp,
            "x_tp": s.dm.x_tp, "w_tp": s.dm.w_tp, "invader": s.dm.invader, "x_sp": s.x_sp, "x_fp": s.x_fp,
            "init_U_sp": s.dm.U_sp.copy(), "init_W_cv": s.dm.W_cv.copy(),
        }
        for d in s.dims:
            out[f"init_BC_fp_{d}"] = getattr(s.dm, f"BC_fp_{d}").copy()
            if s.update == "FV":
                out[f"init_BC_fv_{d}"] = getattr(s.dm, f"BC_fv_{d}").copy()
        if s.potential:
            out["grad_phi_sp"] = s.dm.grad_phi_sp.copy()
            out["grad_phi_fv"] = s.dm.grad_phi_fv.copy()
        out.update(eq_arrays(s))
        limited = s.update == "FV" and s.FB
        s.init_sim()
        dts, crcs, counts = [], [], []
        if "steps" in run:
            # perform_iterations (src/sdader_simulator.py:394-399)
            for _ in range(run["steps"]):
                s.compute_dt()
                dts.append(float(s.dm.dt))
                s.perform_update()
                if limited:
                    c, n = _trouble_digest(s)
                    crcs.append(c)
                    counts.append(n)
        else:
            # perform_time_evolution (src/sdader_simulator.py:401-413)
            t_end = run["t_end"]
            while s.time < t_end:
                s.compute_dt()
                if s.time + s.dm.dt >= t_end:
                    s.dm.dt = t_end - s.time
                if s.dm.dt < 1E-14:
                    break
                dts.append(float(s.dm.dt))
                s.perform_update()
                if limited:
                    c, n = _trouble_digest(s)
                    crcs.append(c)
                    counts.append(n)
        if limited:
            out["troubles"] = s.dm.troubles.copy()
            out["theta"] = s.dm.theta.copy()
            for d in s.dims:
                out[f"affected_faces_{d}"] = getattr(s.dm, f"affected_faces_{d}").copy()
            out["troubles_crc32"] = np.array(crcs, dtype=np.uint32)
            out["troubles_count"] = np.array(counts)
        s.end_sim()
        out["dts"] = np.array(dts)
        out["time"] = np.array(s.time)
        out["n_step"] = np.array(s.n_step)
        for key in ("U_sp", "W_cv"):
            a = np.ascontiguousarray(getattr(s.dm, key))
            if run.get("digest_state"):
                import zlib
                out[f"{key}_crc32"] = np.array(zlib.crc32(a.tobytes()), dtype=np.uint32)
                out[f"{key}_sum"] = np.array(np.sum(a))
                out[f"{key}_absmax"] = np.array(np.max(np.abs(a)))
            else:
                out[key] = a.copy()
        meta = dict(kwargs={k: (list(map(list, v)) if k == "BC" else (list(v) if isinstance(v, tuple) else v))
                            for k, v in kw.items()},
                    ic=list(icspec), run=run, steps=len(dts))
        if icspec[0] == "vortex" and "t_end" in run:
            # exact solution: the vortex translated by (1, 1) * t_end
            shift = 1.0 * run["t_end"]
            exact_fct = ics.isentropic_vortex(center=(5.0 + shift, 5.0 + shift))
            exact = s.crop(rpoly.quadrature_mean(s.mesh_cv, exact_fct, s.ndim, 0)[None])[0]
            out["l1_density_error_vs_exact"] = np.array(np.mean(np.abs(s.dm.W_cv[0] - exact)))
            meta["l1_density_error_vs_exact"] = float(out["l1_density_error_vs_exact"])
        out["case_json"] = np.array(json.dumps(meta))
        path = os.path.join(out_dir, f"{name}.npz")
        np.savez_compressed(path, **out)
        print(name, "steps", len(dts), "time", s.time, "troubles", counts[-1] if counts else "-",
              os.path.getsize(path) // 1024, "KB", flush=True)


if __name__ == "__main__":
    import argparse
    ap = argparse.ArgumentParser()
    ap.add_argument("reference", help="root of the reference's sources (the directory holding src/)")
    ap.add_argument("--only", default="", help="comma-separated case names")
    ap.add_argument("--long", action="store_true", help="make the long-horizon fixtures in long/")
    a = ap.parse_args()
    main(a.reference, only=set(filter(None, a.only.split(","))), long=a.long)
