"""Helpers shared by the GPU parity tests."""
from __future__ import annotations

import numpy as np

DIMS = ("x", "y", "z")


def product_from_golden(data, kw, meta):
    """The product simulator with a golden case's constants and initial state."""
    from golden_cases import golden_operators, make_ic
    from spd_gb300 import SDADER_Simulator
    s = SDADER_Simulator(init_fct=make_ic(meta["ic"]), operators=golden_operators(data), verbose=False, **kw)
    s.dm.U_sp = data["init_U_sp"]
    # long-horizon fixtures carry no initial U_cv: the step never reads it
    # before recomputing it from U_sp (FV) or at the end of a run (SD)
    s.dm.U_cv = data["init_U_cv"] if "init_U_cv" in data else s.compute_conservatives(data["init_W_cv"])
    s.dm.W_cv = data["init_W_cv"]
    # the stored boundary arrays of the reference's run (the "ic", "eq" and
    # "pressure" sides read them; made here they would carry this machine's
    # einsum roundings)
    for d in s.dims:
        if f"init_BC_fp_{d}" in data:
            s._ctx.upload(f"BC_fp_{d}", data[f"init_BC_fp_{d}"])
        if f"init_BC_fv_{d}" in data and s.update == "FV":
            s._ctx.upload(f"BC_fv_{d}", data[f"init_BC_fv_{d}"])
    if kw.get("potential", False):
        s.dm.grad_phi_sp = data["grad_phi_sp"]
        s.dm.grad_phi_fv = data["grad_phi_fv"]
    if kw.get("WB", False):
        s.upload_equilibrium({name: data[name] for name in wb_fields(s) if name in data})
    return s


def wb_fields(s):
    """Names of the well-balanced mode's equilibrium arrays for ``s``."""
    from golden_cases import WB_KEYS
    names = []
    for key in WB_KEYS:
        names += [key] if key in ("U_eq_sp", "U_eq_cv", "M_eq_fv") else [f"{key}_{d}" for d in s.dims]
    return [n for n in names if s.update == "FV" or not (n.startswith("M_eq_faces") or
                                                          n.startswith("F_eq_faces") or n == "M_eq_fv")]


def oracle_like(s, **override):
    """An oracle run with the same constants and initial state as the
    product simulator ``s`` (state downloaded from the device)."""
    from oracle.sdader_oracle import OracleSDADER
    ndim = s.ndim
    state = {"U_sp": s.dm.U_sp, "U_cv": s.dm.U_cv, "W_cv": s.dm.W_cv}
    T = s.nader
    for dim in s.dims:
        idim = s.dims[dim]
        M_fp = s.compute_fp_from_sp(state["U_sp"], dim)
        first = [slice(None)] * M_fp.ndim
        last = [slice(None)] * M_fp.ndim
        first[-(ndim + idim + 1)] = 0
        first[-(idim + 1)] = 0
        last[-(ndim + idim + 1)] = -1
        last[-(idim + 1)] = -1
        state[f"BC_fp_{dim}"] = np.stack([np.repeat(M_fp[tuple(first)][:, None], T, axis=1),
                                          np.repeat(M_fp[tuple(last)][:, None], T, axis=1)])
        if s.update == "FV":
            ext = [s.N[DIMS[i]] * s.n[DIMS[i]] + 2 * s.Nghc for i in range(ndim)]
            ext[idim] = s.Nghc
            state[f"BC_fv_{dim}"] = s._ctx.download(f"BC_fv_{dim}", (2, s.nvar) + tuple(ext[::-1]))
    kw = dict(ndim=ndim, N=[s.N[d] for d in s.dims], p=s.p, m=s.m, lims=[s.lim[d] for d in s.dims],
              BC=[s.BC[d] for d in s.dims], gamma=s.gamma, cfl_coeff=s.cfl_coeff, min_c2=s.min_c2,
              riemann_solver_sd=s.riemann_solver_sd_name, riemann_solver_fv=s.riemann_solver_fv_name,
              slope_limiter=s.slope_limiter_name, update=s.update, FB=s.FB, tolerance=s.tolerance, SED=s.SED,
              NAD=s.NAD, PAD=s.PAD, blending=s.blending, min_rho=s.min_rho, max_rho=s.max_rho, min_P=s.min_P,
              godunov=s.godunov, ops=s.ops, state=state, viscosity=s.viscosity, nu=s.nu, beta=s.beta,
              potential=s.potential, isothermal=s.isothermal, WB=s.WB)
    if s.potential:
        state["grad_phi_sp"] = s.dm.grad_phi_sp
        state["grad_phi_fv"] = s.dm.grad_phi_fv
    if s.WB:
        for name in wb_fields(s):
            state[name] = getattr(s.dm, name)
    kw.update(override)
    return OracleSDADER(**kw)


def step_both(s, o, nsteps):
    """Advance product and oracle by nsteps (compute_dt + perform_update);
    returns the list of (dt_product, dt_oracle)."""
    dts = []
    for _ in range(nsteps):
        s.compute_dt()
        o.compute_dt()
        dts.append((s.dm.dt, o.dt))
        s.perform_update()
        o.perform_update()
    return dts


def compare(s, o, check_masks=True):
    """Bitwise comparison of the product state with the oracle's; returns a
    dict of mismatching fields with the max relative deviation."""
    bad = {}
    for key, ref in (("U_sp", o.U_sp), ("U_cv", o.U_cv), ("W_cv", o.W_cv)):
        got = getattr(s.dm, key)
        if not np.array_equal(got, ref, equal_nan=True):
            bad[key] = float(np.nanmax(np.abs(got - ref) / np.maximum(np.abs(ref), 1e-300)))
    if check_masks and s.update == "FV" and s.FB and o.troubles is not None:
        if not np.array_equal(s.dm.troubles, o.troubles):
            bad["troubles"] = int(np.sum(s.dm.troubles != o.troubles))
        if not np.array_equal(s.dm.theta, o.theta, equal_nan=True):
            bad["theta"] = int(np.sum(s.dm.theta != o.theta))
        for i, dim in enumerate(s.dims):
            if not np.array_equal(getattr(s.dm, f"affected_faces_{dim}"), o.affected[i], equal_nan=True):
                bad[f"affected_faces_{dim}"] = 1
    return bad
