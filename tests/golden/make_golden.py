"""Generate the golden fixtures in this directory by running the reference.

Run once in a container where the reference's sources are present:

    python tests/golden/make_golden.py /path/to/reference

It imports the reference's NumPy implementation (``src/`` of jpalafou/spd,
CuPy absent so the FP64 NumPy path runs), builds each case below, records
the constant operators and the initial state, advances the listed number of
steps with ``compute_dt`` + ``perform_update`` (the body of
``perform_iterations``) and records the state after every case.  The
fixtures are .npz files; ``case.json`` inside each describes the run.
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
}


def make_ic(spec):
    name, kw = spec
    if name == "vortex":
        return ics.isentropic_vortex()
    if name in ("sedov", "kelvin_helmholtz"):
        return getattr(ics, name)(**kw)
    return getattr(ics, name)


def main(ref_root):
    sys.path.insert(0, os.path.join(ref_root, "src"))
    warnings.simplefilter("ignore")
    from sdader_simulator import SDADER_Simulator  # the reference
    import polynomials as rpoly

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
        init = make_ic(icspec)
        s = SDADER_Simulator(init_fct=init, use_cupy=False, verbose=False, **kw)
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
        s.init_sim()
        dts = []
        for _ in range(steps):
            s.compute_dt()
            dts.append(float(s.dm.dt))
            s.perform_update()
        out["dts"] = np.array(dts)
        out["time"] = np.array(s.time)
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


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else "/root/reference")
