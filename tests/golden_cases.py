"""Load the golden fixtures (outputs of the reference's NumPy path) and
build matching oracle / product runs from them."""
from __future__ import annotations

import glob
import json
import os

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
DIMS = ("x", "y", "z")


LONG = os.path.join(GOLDEN, "long")
# equilibrium arrays of the well-balanced mode in a fixture
WB_KEYS = ("U_eq_sp", "U_eq_cv", "M_eq_fp", "F_eq_fp", "M_eq_faces", "F_eq_faces", "M_eq_fv")


def long_case_names():
    return sorted(os.path.splitext(os.path.basename(p))[0] for p in glob.glob(os.path.join(LONG, "*.npz")))


def case_names():
    return sorted(os.path.splitext(os.path.basename(p))[0] for p in glob.glob(os.path.join(GOLDEN, "*.npz"))
                  if not p.endswith("operators.npz"))


def adjoint_case_names():
    """The golden cases the adjoint covers: not viscosity, gravity, the
    isothermal system or the well-balanced mode (spd_adjoint_enable refuses
    those)."""
    out = []
    for name in case_names():
        kw = load(name)[1]
        if not (kw.get("viscosity") or kw.get("potential") or kw.get("isothermal") or kw.get("WB")):
            out.append(name)
    return out


def load_long(name):
    """A long-horizon fixture: as ``load``; ``meta["run"]`` is {"steps": n}
    or {"t_end": t}, and the arrays hold the dt of every step and, with
    limiting, a CRC-32 and count of the trouble mask after every step."""
    return load(name, LONG)


def load(name, where=GOLDEN):
    z = np.load(os.path.join(where, f"{name}.npz"))
    data = {k: z[k] for k in z.files}
    meta = json.loads(str(data.pop("case_json")))
    kw = dict(meta["kwargs"])
    if "N" in kw:
        kw["N"] = tuple(kw["N"])
    for key in ("xlim", "ylim", "zlim"):
        if key in kw:
            kw[key] = tuple(kw[key])
    kw["BC"] = tuple(tuple(b) for b in kw["BC"])
    if "eq_ic" in kw:
        # the equilibrium of the well-balanced mode, as a callback
        kw["eq_fct"] = make_ic(tuple(kw.pop("eq_ic")))
    return data, kw, meta


def make_ic(spec):
    from spd_gb300 import initial_conditions as ics
    name, kw = spec
    if name == "vortex":
        return ics.isentropic_vortex()
    if name in ("sedov", "kelvin_helmholtz", "gravity_column"):
        return getattr(ics, name)(**kw)
    return getattr(ics, name)


def oracle_from_golden(data, kw):
    from oracle.sdader_oracle import OracleSDADER
    ndim = len(kw["N"])
    p = kw["p"]
    lims = [kw.get(f"{d}lim", (0, 1)) for d in DIMS[:ndim]]
    ops = {k: data[k] for k in ("sp_to_fp", "dfp_to_sp", "sp_to_cv", "cv_to_sp", "w_tp", "invader", "x_fp")}
    from oracle.sdader_oracle import compute_conservatives
    # long-horizon fixtures carry no initial U_cv: the step never reads it
    # before recomputing it from U_sp (FV) or at the end of a run (SD)
    U_cv = data["init_U_cv"] if "init_U_cv" in data else compute_conservatives(data["init_W_cv"], ndim,
                                                                                 kw.get("gamma", 1.4))
    state = {"U_sp": data["init_U_sp"], "U_cv": U_cv, "W_cv": data["init_W_cv"]}
    if kw.get("potential", False):
        state["grad_phi_sp"] = data["grad_phi_sp"]
        state["grad_phi_fv"] = data["grad_phi_fv"]
    for key in WB_KEYS:
        for name in (key, *(f"{key}_{d}" for d in DIMS[:ndim])):
            if name in data:
                state[name] = data[name]
    for d in DIMS[:ndim]:
        state[f"BC_fp_{d}"] = data[f"init_BC_fp_{d}"]
        if f"init_BC_fv_{d}" in data:
            state[f"BC_fv_{d}"] = data[f"init_BC_fv_{d}"]
    return OracleSDADER(
        ndim=ndim, N=list(kw["N"]), p=p, m=kw.get("m", -1) if kw.get("m", -1) != -1 else p, lims=lims,
        BC=kw["BC"], gamma=kw.get("gamma", 1.4), cfl_coeff=kw.get("cfl_coeff", 0.8), min_c2=kw.get("min_c2", 1e-10),
        riemann_solver_sd=kw.get("riemann_solver_sd", "llf"), riemann_solver_fv=kw.get("riemann_solver_fv", "llf"),
        slope_limiter=kw.get("slope_limiter", "minmod"), update=kw.get("update", "SD"), FB=kw.get("FB", False),
        tolerance=kw.get("tolerance", 1e-5), SED=kw.get("SED", True), NAD=kw.get("NAD", ""),
        PAD=kw.get("PAD", True), blending=kw.get("blending", True), min_rho=kw.get("min_rho", 1e-10),
        max_rho=kw.get("max_rho", 1e10), min_P=kw.get("min_P", 1e-10), godunov=kw.get("godunov", False),
        ops=ops, state=state, viscosity=kw.get("viscosity", False), nu=kw.get("nu", 1e-4),
        beta=kw.get("beta", 2.0 / 3), potential=kw.get("potential", False),
        isothermal=kw.get("isothermal", False), WB=kw.get("WB", False))


def golden_operators(data):
    return {k: data[k] for k in ("sp_to_fp", "fp_to_sp", "dfp_to_sp", "sp_to_cv", "fp_to_cv", "cv_to_sp",
                                 "x_tp", "w_tp", "invader", "x_sp", "x_fp")}


def trouble_digest(troubles):
    """CRC-32 of the trouble mask's bytes and its count (the per-step pin of
    the long-horizon fixtures)."""
    import zlib
    t = np.ascontiguousarray(np.asarray(troubles, dtype=np.float64))
    return zlib.crc32(t.tobytes()), float(t.sum())


def run_like_reference(sim, meta, limited, get_dt, set_dt, get_time, troubles):
    """Advance ``sim`` (product or oracle) exactly as the reference's
    perform_iterations / perform_time_evolution loops do (without their
    end_sim); returns the dts and the per-step trouble digests."""
    run = meta["run"]
    dts, crcs, counts = [], [], []

    def after():
        if limited:
            c, n = trouble_digest(troubles())
            crcs.append(c)
            counts.append(n)

    if "steps" in run:
        for _ in range(run["steps"]):
            sim.compute_dt()
            dts.append(get_dt())
            sim.perform_update()
            after()
    else:
        t_end = run["t_end"]
        while get_time() < t_end:
            sim.compute_dt()
            if get_time() + get_dt() >= t_end:
                set_dt(t_end - get_time())
            if get_dt() < 1E-14:
                break
            dts.append(get_dt())
            sim.perform_update()
            after()
    return dts, crcs, counts


def state_matches(got, data, key):
    """Bitwise comparison of a final state array with a fixture that holds
    either the array or the CRC-32 digest of its bytes; returns (ok, info)."""
    got = np.ascontiguousarray(np.asarray(got, dtype=np.float64))
    if key in data:
        ok = np.array_equal(got, data[key], equal_nan=True)
        return ok, (None if ok else float(np.nanmax(np.abs(got - data[key]))))
    import zlib
    crc = zlib.crc32(got.tobytes())
    ok = crc == int(data[f"{key}_crc32"])
    return ok, (None if ok else (float(np.sum(got)), float(data[f"{key}_sum"]),
                                 float(np.max(np.abs(got))), float(data[f"{key}_absmax"])))
