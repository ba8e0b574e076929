"""CPU oracle for the SD-ADER step of jpalafou/spd -- TEST INFRASTRUCTURE ONLY.

This module is a NumPy FP64 restatement of the reference's SD-ADER time step
(predictor, SD update, subcell finite-volume update with a-posteriori
limiting).  It exists to check the CUDA path: only ``tests/``,
``__graft_entry__.smoke()`` and the CPU-baseline leg of ``bench.py`` may
import it.  The product (``spd_gb300``) never calls it.

Parity pin: every function follows the reference file:line cited in its
docstring, with the same operation order and the same intermediate
roundings.  Contractions do not call ``np.einsum``; they sum in the order
NumPy 2.5's einsum uses on the x86_64 machine where the golden fixtures were
made (a two-lane accumulation when the contracted axis is the contiguous
last axis, a plain left-to-right sum otherwise; see ``_sum_terms``).  The
restatement is pinned bit-for-bit against the reference's own outputs in
``tests/golden/`` (made by ``tests/golden/make_golden.py``, which imports
the reference itself).

Layouts are the reference's: SD arrays are (V, [T], Nz, Ny, Nx, nz, ny, nx)
with absent dimensions dropped, FV arrays are (V, Nz*n, Ny*n, Nx*n).
"""
from __future__ import annotations

import numpy as np

DIMS = ("x", "y", "z")


# ----------------------------------------------------------------------------
# summation order of the reference's contractions
# ----------------------------------------------------------------------------
def _sum_terms(terms, order):
    """Sum a list of arrays in a fixed order.

    ``seq``: ((t0 + t1) + t2) + ...  -- einsum over a strided axis
    (src/transforms.py:8-10 for y/z, the Picard einsum
    src/sdader_simulator.py:196 and the weighted sum :205).
    ``lanes2``: (t0 + t2 + t4 ...) + (t1 + t3 + ...) -- einsum over the
    contiguous last axis (src/transforms.py:5, the x direction).
    """
    if order == "seq":
        acc = terms[0]
        for t in terms[1:]:
            acc = acc + t
        return acc
    even = terms[0]
    odd = None
    for s in range(1, len(terms)):
        if s % 2 == 0:
            even = even + terms[s]
        elif odd is None:
            odd = terms[s]
        else:
            odd = odd + terms[s]
    return even if odd is None else even + odd


def apply_axis(A, M, axis, order):
    """out[..., f, ...] = sum_s A[f, s] * M[..., s, ...] along ``axis``.

    Restates ``compute_A_from_B`` (src/transforms.py:3-25).
    """
    axis = axis % M.ndim
    n_to, n_from = A.shape
    assert M.shape[axis] == n_from
    outs = []
    for f in range(n_to):
        terms = [A[f, s] * np.take(M, s, axis=axis) for s in range(n_from)]
        outs.append(_sum_terms(terms, order))
    return np.stack(outs, axis=axis)


def apply_full(A, M, ndim, rows=False):
    """Apply the 1D operator along every one of the last ``ndim`` axes at once.

    Restates ``compute_A_from_B_full`` (src/transforms.py:27-45).  Products
    are formed as ((A*A)*A)*M.  For a C-contiguous input (every call except
    the one in ``switch_to_high_order``) einsum sums all input points in one
    row-major sequence; 1D uses the contiguous two-lane sum, and 2D with two
    points per axis pairs the rows.  For the strided SD view of an FV array
    (src/sdader_simulator.py:302-307, ``rows=True``) each row along the last
    axis is summed on its own and the row sums are then added in order.
    """
    n = A.shape[1]
    if ndim == 1:
        return apply_axis(A, M, -1, "lanes2")
    if ndim == 2:
        out = np.empty(M.shape[:-2] + (A.shape[0], A.shape[0]))
        for j in range(A.shape[0]):
            for i in range(A.shape[0]):
                if rows or n == 2:
                    row_sums = [_sum_terms([(A[j, m] * A[i, l]) * M[..., m, l] for l in range(n)], "seq")
                                for m in range(n)]
                    out[..., j, i] = _sum_terms(row_sums, "seq")
                else:
                    terms = [(A[j, m] * A[i, l]) * M[..., m, l]
                             for m in range(n) for l in range(n)]
                    out[..., j, i] = _sum_terms(terms, "seq")
        return out
    out = np.empty(M.shape[:-3] + (A.shape[0],) * 3)
    for k in range(A.shape[0]):
        for j in range(A.shape[0]):
            for i in range(A.shape[0]):
                if rows:
                    row_sums = [_sum_terms([((A[k, a] * A[j, b]) * A[i, c]) * M[..., a, b, c]
                                            for c in range(n)], "seq")
                                for a in range(n) for b in range(n)]
                    out[..., k, j, i] = _sum_terms(row_sums, "seq")
                else:
                    terms = [((A[k, a] * A[j, b]) * A[i, c]) * M[..., a, b, c]
                             for a in range(n) for b in range(n) for c in range(n)]
                    out[..., k, j, i] = _sum_terms(terms, "seq")
    return out


def sp_axis(ndim, idim):
    """Array axis (negative) of the in-cell point index for dimension idim."""
    return -(idim + 1)


def cell_axis(ndim, idim):
    """Array axis (negative) of the cell index for dimension idim."""
    return -(ndim + idim + 1)


def axis_order(idim):
    """x contracts over the contiguous last axis; y and z do not."""
    return "lanes2" if idim == 0 else "seq"


# ----------------------------------------------------------------------------
# hydro (src/hydro.py)
# ----------------------------------------------------------------------------
def compute_primitives(U, ndim, gamma, vels=None):
    """src/hydro.py:48-86 (U -> W); the kinetic term sums in ``vels`` order."""
    W = U.copy()
    _p_ = ndim + 1
    K = None
    for vel in (range(1, ndim + 1) if vels is None else vels):
        W[vel] = U[vel] / U[0]
        K = W[vel] * W[vel] if K is None else K + W[vel] * W[vel]
    K = K * (0.5 * U[0])
    W[_p_] = (gamma - 1) * (U[_p_] - K)
    return W


def compute_conservatives(W, ndim, gamma, vels=None):
    """src/hydro.py:88-125 (W -> U); the kinetic term sums in ``vels`` order."""
    U = W.copy()
    _p_ = ndim + 1
    K = None
    for vel in (range(1, ndim + 1) if vels is None else vels):
        U[vel] = W[vel] * U[0]
        K = W[vel] * W[vel] if K is None else K + W[vel] * W[vel]
    K = K * (0.5 * U[0])
    U[_p_] = W[_p_] / (gamma - 1) + K
    return U


def compute_fluxes(W, vels, gamma):
    """src/hydro.py:127-170; ``vels`` is the rotated velocity index list."""
    ndim = len(vels)
    _p_ = ndim + 1
    F = np.empty_like(W)
    v1 = vels[0]
    K = None
    m = None
    for v in vels[::-1]:
        m = W[0] * W[v]
        K = m * W[v] if K is None else K + m * W[v]
        F[v] = m * W[v1]
    E = W[_p_] / (gamma - 1) + 0.5 * K
    F[0] = m
    F[v1] = m * W[v1] + W[_p_]
    F[_p_] = W[v1] * (E + W[_p_])
    return F


def compute_cs(P, rho, gamma, min_c2):
    """src/hydro.py:3-46: sqrt of gamma*P/rho floored at min_c2 (NaN -> floor)."""
    c2 = gamma * P / rho
    c2 = np.where(c2 > min_c2, c2, min_c2)
    return np.sqrt(c2)


# ----------------------------------------------------------------------------
# Riemann solvers (src/riemann_solver.py)
# ----------------------------------------------------------------------------
def riemann(name, M_L, M_R, vels, gamma, min_c2, prims):
    """src/riemann_solver.py:10-29 wrapper, then llf/hllc/lhllc."""
    ndim = len(vels)
    if prims:
        W_L, W_R = M_L, M_R
        U_L = compute_conservatives(W_L, ndim, gamma, vels)
        U_R = compute_conservatives(W_R, ndim, gamma, vels)
    else:
        U_L, U_R = M_L, M_R
        W_L = compute_primitives(U_L, ndim, gamma, vels)
        W_R = compute_primitives(U_R, ndim, gamma, vels)
    if name == "llf":
        return _llf(W_L, W_R, U_L, U_R, vels, gamma, min_c2)
    if name in ("hllc", "lhllc"):
        return _hllc(W_L, W_R, U_L, U_R, vels, gamma, min_c2, low_mach=(name == "lhllc"))
    raise AttributeError(name)


def _llf(W_L, W_R, U_L, U_R, vels, gamma, min_c2):
    """src/riemann_solver.py:31-65."""
    _p_ = len(vels) + 1
    v1 = vels[0]
    F_L = compute_fluxes(W_L, vels, gamma)
    F_R = compute_fluxes(W_R, vels, gamma)
    c_L = compute_cs(W_L[_p_], W_L[0], gamma, min_c2) + np.abs(W_L[v1])
    c_R = compute_cs(W_R[_p_], W_R[0], gamma, min_c2) + np.abs(W_R[v1])
    c_max = np.where(c_L > c_R, c_L, c_R)[np.newaxis, ...]
    return 0.5 * (F_R + F_L) - 0.5 * c_max * (U_R - U_L)


def _hllc(W_L, W_R, U_L, U_R, vels, gamma, min_c2, low_mach=False):
    """src/riemann_solver.py:67-145 (hllc) and :147-212 (lhllc)."""
    _p_ = len(vels) + 1
    v1 = vels[0]
    c_L = compute_cs(W_L[_p_], W_L[0], gamma, min_c2) + np.abs(W_L[v1])
    c_R = compute_cs(W_R[_p_], W_R[0], gamma, min_c2) + np.abs(W_R[v1])
    c_max = np.where(c_L > c_R, c_L, c_R)
    v_L = W_L[v1]
    v_R = W_R[v1]
    s_L = np.where(v_L < v_R, v_L, v_R) - c_max
    s_R = np.where(v_L > v_R, v_L, v_R) + c_max
    rc_L = W_L[0] * (v_L - s_L)
    rc_R = W_R[0] * (s_R - v_R)
    with np.errstate(all="ignore"):
        v_star = (rc_R * v_R + rc_L * v_L + (W_L[_p_] - W_R[_p_])) / (rc_R + rc_L)
        if low_mach:
            Mach = np.minimum(1, np.maximum(np.abs(v_L), np.abs(v_R)) / c_max)
            phi = Mach * (2 - Mach)
            P_star = (rc_R * W_L[_p_] + rc_L * W_R[_p_] + phi * rc_L * rc_R * (v_L - v_R)) / (rc_R + rc_L)
        else:
            P_star = (rc_R * W_L[_p_] + rc_L * W_R[_p_] + rc_L * rc_R * (v_L - v_R)) / (rc_R + rc_L)
        r_starL = W_L[0] * (s_L - v_L) / (s_L - v_star)
        e_starL = ((s_L - v_L) * U_L[_p_] - W_L[_p_] * v_L + P_star * v_star) / (s_L - v_star)
        r_starR = W_R[0] * (s_R - v_R) / (s_R - v_star)
        e_starR = ((s_R - v_R) * U_R[_p_] - W_R[_p_] * v_R + P_star * v_star) / (s_R - v_star)
    r_gdv = np.where(s_L > 0, W_L[0], np.where(v_star > 0, r_starL, np.where(s_R > 0, r_starR, W_R[0])))
    v_gdv = np.where(s_L > 0, v_L, np.where(v_star > 0, v_star, np.where(s_R > 0, v_star, v_R)))
    P_gdv = np.where(s_L > 0, W_L[_p_], np.where(v_star > 0, P_star, np.where(s_R > 0, P_star, W_R[_p_])))
    e_gdv = np.where(s_L > 0, U_L[_p_], np.where(v_star > 0, e_starL, np.where(s_R > 0, e_starR, U_R[_p_])))
    F = np.empty_like(W_L)
    F[0] = r_gdv * v_gdv
    F[v1] = F[0] * v_gdv + P_gdv
    F[_p_] = v_gdv * (e_gdv + P_gdv)
    for vel in vels[1:]:
        F[vel] = F[0] * np.where(v_star > 0, W_L[vel], W_R[vel])
    return F


# ----------------------------------------------------------------------------
# slope limiters and MUSCL-Hancock (src/muscl.py)
# ----------------------------------------------------------------------------
def _shift(M, start, end, axis):
    sl = [slice(None)] * M.ndim
    sl[axis] = slice(start, end)
    return M[tuple(sl)]


def minmod(SL, SR):
    """src/muscl.py:12-35 (ratio form; NaN ratio -> 0)."""
    with np.errstate(all="ignore"):
        ratio = SR / SL
    ratio = np.where(ratio < 1, ratio, 1)
    return np.where(ratio > 0, ratio, 0) * SL


def moncen(dU_L, dU_R, dx_L, dx_R, dx_M):
    """src/muscl.py:37-59."""
    dU_C = (dx_L * dU_L + dx_R * dU_R) / (dx_L + dx_R)
    slope = np.minimum(np.abs(2 * dU_L * dx_L / dx_M), np.abs(2 * dU_R * dx_R / dx_M))
    slope = np.sign(dU_C) * np.minimum(slope, np.abs(dU_C))
    return np.where(dU_L * dU_R >= 0, slope, 0)


def limited_gradient(M, h_cv, h_fp, axis, limiter):
    """src/muscl.py:61-75 along array axis ``axis`` (h arrays broadcast)."""
    dM = (_shift(M, 1, None, axis) - _shift(M, None, -1, axis)) / h_cv
    SL = _shift(dM, None, -1, axis)
    SR = _shift(dM, 1, None, axis)
    if limiter == "minmod":
        return minmod(SL, SR)
    return moncen(SL, SR, _shift(h_cv, None, -1, axis), _shift(h_cv, 1, None, axis),
                  _shift(h_fp, 1, -1, axis))


# ----------------------------------------------------------------------------
# setup-time geometry (src/sdader_simulator.py:61-92)
# ----------------------------------------------------------------------------
def subcell_faces(N, h, fp_ref, ngh):
    """Subcell face positions with ngh mirrored ghost faces per side."""
    n = len(fp_ref) - 1
    fp = np.empty(N * n + 2 * ngh + 1)
    fp[ngh:-ngh] = h * np.hstack((np.arange(N).repeat(n) + np.tile(fp_ref[:-1], N), N))
    fp[:ngh] = -fp[(ngh + 1):(2 * ngh + 1)][::-1]
    fp[-ngh:] = fp[-(ngh + 1)] + fp[ngh + 1:2 * ngh + 1]
    return fp


# ----------------------------------------------------------------------------
# the simulator restatement
# ----------------------------------------------------------------------------
class OracleSDADER:
    """Restates ``SDADER_Simulator``'s step (src/sdader_simulator.py:14-476).

    ``ops`` holds the constant operators built at setup
    (src/sd_simulator.py:30-52, src/sdader_simulator.py:40-46):
    keys sp_to_fp, dfp_to_sp, sp_to_cv, cv_to_sp, w_tp, invader, x_fp.
    ``state`` holds U_sp, U_cv, W_cv (SD layout) and the initial boundary
    arrays BC_fp_<dim> (for "ic"/"eq"/"pressure" sides) and BC_fv_<dim>.
    """

    def __init__(self, *, ndim, N, p, m, lims, BC, gamma, cfl_coeff, min_c2,
                 riemann_solver_sd, riemann_solver_fv, slope_limiter, update,
                 FB, tolerance, SED, NAD, PAD, blending, min_rho, max_rho,
                 min_P, godunov, ops, state, Nghc=2):
        self.ndim = ndim
        self.N = list(N)          # cells per dim, x first
        self.p = p
        self.m = m
        self.n = p + 1
        self.nf = p + 2
        self.T = m + 1
        self.V = ndim + 2
        self.BC = [tuple(BC[i]) for i in range(ndim)]
        self.gamma = gamma
        self.cfl = cfl_coeff
        self.min_c2 = min_c2
        self.rs_sd = riemann_solver_sd
        self.rs_fv = riemann_solver_fv
        self.limiter = slope_limiter
        self.update = update
        self.FB = FB
        self.tol = tolerance
        self.SED = SED
        self.NAD = NAD
        self.PAD = PAD
        self.blending = blending
        self.min_rho = min_rho
        self.max_rho = max_rho
        self.min_P = min_P
        self.godunov = godunov
        self.ngh = Nghc
        self.ops = ops
        self.h = [(lims[i][1] - lims[i][0]) / self.N[i] for i in range(ndim)]
        self.h_min = 1e10
        for hh in self.h:
            self.h_min = min(self.h_min, hh)
        self.U_sp = state["U_sp"].copy()
        self.U_cv = state["U_cv"].copy()
        self.W_cv = state["W_cv"].copy()
        self.BC_fp = {i: state[f"BC_fp_{DIMS[i]}"].copy() for i in range(ndim)}
        self.BC_fv = {i: state[f"BC_fv_{DIMS[i]}"].copy() for i in range(ndim)
                      if f"BC_fv_{DIMS[i]}" in state}
        self.time = 0.0
        self.n_step = 0
        self.dt = None
        # subcell geometry (src/sdader_simulator.py:61-92)
        self.faces, self.centers, self.h_fp, self.h_cv = [], [], [], []
        for i in range(ndim):
            fp = subcell_faces(self.N[i], self.h[i], ops["x_fp"], self.ngh)
            cv = 0.5 * (fp[1:] + fp[:-1])
            self.faces.append(fp)
            self.centers.append(cv)
            self.h_fp.append(fp[1:] - fp[:-1])
            self.h_cv.append(cv[1:] - cv[:-1])
        self.troubles = None
        self.theta = None
        self.affected = {}

    # ---- helpers --------------------------------------------------------
    def vels(self):
        return list(range(1, self.ndim + 1))

    def rolled_vels(self, idim):
        return list(np.roll(np.arange(1, self.ndim + 1), -idim))

    def bshape(self, arr, idim, nd=None):
        """Broadcast a 1D array along FV axis idim of an nd-dim spatial array."""
        nd = self.ndim if nd is None else nd
        shp = [1] * nd
        shp[nd - 1 - idim] = -1
        return arr.reshape(shp)

    # ---- dt (src/sd_simulator.py:214-227) --------------------------------
    def compute_dt(self):
        W = self.W_cv
        _p_ = self.ndim + 1
        c_s = compute_cs(W[_p_], W[0], self.gamma, self.min_c2)
        c = c_s * self.ndim
        for vel in self.vels():
            c = c + np.abs(W[vel])
        c_max = np.max(c)
        h = self.h_min / (self.p + 1)
        dt = h / c_max
        self.dt = self.cfl * dt
        return self.dt

    # ---- predictor (src/sdader_simulator.py:160-240) ---------------------
    def solve_faces(self, U_ader):
        """Returns F_ader_fp per dim with Riemann fluxes at element edges."""
        ops = self.ops
        nd = self.ndim
        F_all = {}
        for idim in range(nd):
            vels = self.rolled_vels(idim)
            ax_sp = sp_axis(nd, idim)
            ax_cell = cell_axis(nd, idim)
            M_fp = apply_axis(ops["sp_to_fp"], U_ader, ax_sp, axis_order(idim))
            F_fp = compute_fluxes(compute_primitives(M_fp, nd, self.gamma), vels, self.gamma)
            # edge traces (src/sd_boundary.py:7-17)
            left_trace = np.take(M_fp, 0, axis=ax_sp)     # fp 0 of every cell
            right_trace = np.take(M_fp, self.nf - 1, axis=ax_sp)
            # axis of cells along idim in the trace arrays (one fewer axis)
            tax = ax_cell + 1
            Ncell = self.N[idim]
            first_l = np.take(left_trace, 0, axis=tax)
            last_r = np.take(right_trace, Ncell - 1, axis=tax)
            bc = []
            for side in (0, 1):
                kind = self.BC[idim][side]
                if kind == "periodic":
                    v = last_r.copy() if side == 0 else first_l.copy()
                elif kind in ("reflective", "gradfree"):
                    v = first_l.copy() if side == 0 else last_r.copy()
                    if kind == "reflective":
                        v[idim + 1] = v[idim + 1] * -1
                elif kind in ("ic", "eq"):
                    v = np.broadcast_to(self.BC_fp[idim][side], first_l.shape).copy()
                elif kind == "pressure":
                    v = np.broadcast_to(self.BC_fp[idim][side], first_l.shape).copy()
                else:
                    raise TypeError("Undetermined boundary type")
                bc.append(v)
            # pressure sides overwrite the edge traces with the stored state
            if self.BC[idim][0] == "pressure":
                left_trace = left_trace.copy()
                idx = [slice(None)] * left_trace.ndim
                idx[tax] = 0
                left_trace[tuple(idx)] = bc[0]
            if self.BC[idim][1] == "pressure":
                right_trace = right_trace.copy()
                idx = [slice(None)] * right_trace.ndim
                idx[tax] = Ncell - 1
                right_trace[tuple(idx)] = bc[1]
            ML = np.concatenate([np.expand_dims(bc[0], tax), right_trace], axis=tax)
            MR = np.concatenate([left_trace, np.expand_dims(bc[1], tax)], axis=tax)
            F = riemann(self.rs_sd, ML, MR, vels, self.gamma, self.min_c2, prims=False)
            # scatter (src/sd_boundary.py:19-30)
            idx0 = [slice(None)] * F_fp.ndim
            idx0[ax_sp] = 0
            F_fp[tuple(idx0)] = _shift(F, None, -1, tax)
            idx1 = [slice(None)] * F_fp.ndim
            idx1[ax_sp] = self.nf - 1
            F_fp[tuple(idx1)] = _shift(F, 1, None, tax)
            F_all[idim] = F_fp
        return F_all

    def ader_dudt(self, F_all):
        """src/sdader_simulator.py:148-158 with src/sd_simulator.py:196-206."""
        dUdt = None
        for idim in range(self.ndim):
            part = apply_axis(self.ops["dfp_to_sp"], F_all[idim], sp_axis(self.ndim, idim),
                              axis_order(idim)) / self.h[idim]
            dUdt = part if dUdt is None else dUdt + part
        return dUdt

    def ader_predictor(self):
        """src/sdader_simulator.py:160-200; returns the last F_ader_fp."""
        T = self.T
        U_ader = np.repeat(self.U_sp[:, np.newaxis], T, axis=1)
        inv = self.ops["invader"]
        F_all = None
        for it in range(self.m + 1):
            F_all = self.solve_faces(U_ader)
            if it < self.m:
                dudt = self.ader_dudt(F_all)
                terms_n = []
                for nn in range(T):
                    terms = [inv[nn, pp] * dudt[:, pp] for pp in range(T)]
                    terms_n.append(_sum_terms(terms, "seq"))
                upd = np.stack(terms_n, axis=1) * self.dt
                U_ader = self.U_sp[:, np.newaxis] - upd
        self.F_ader = F_all
        return F_all

    def ader_update(self, F_all):
        """src/sdader_simulator.py:202-208."""
        dudt = self.ader_dudt(F_all)
        w = self.ops["w_tp"]
        terms = [w[t] * dudt[:, t] for t in range(self.T)]
        dUdt = _sum_terms(terms, "seq") * self.dt
        self.U_sp = self.U_sp - dUdt

    # ---- SD <-> FV layouts (src/sd_simulator.py:104-131) -----------------
    def to_fv(self, M):
        nd = self.ndim
        if nd == 1:
            return M.reshape(M.shape[0], M.shape[1] * M.shape[2])
        if nd == 2:
            return np.transpose(M, (0, 1, 3, 2, 4)).reshape(
                M.shape[0], M.shape[1] * M.shape[3], M.shape[2] * M.shape[4])
        return np.transpose(M, (0, 1, 4, 2, 5, 3, 6)).reshape(
            M.shape[0], M.shape[1] * M.shape[4], M.shape[2] * M.shape[5], M.shape[3] * M.shape[6])

    def to_sd(self, M):
        nd = self.ndim
        shape = []
        for i in range(nd):
            shape += [self.n, self.N[i]]
        shape = [M.shape[0]] + shape[::-1]
        if nd == 1:
            return M.reshape(shape)
        if nd == 2:
            return np.transpose(M.reshape(shape), (0, 1, 3, 2, 4))
        return np.transpose(M.reshape(shape), (0, 1, 3, 5, 2, 4, 6))

    # ---- FV machinery (src/fv_simulator.py, src/trouble_detection.py) ----
    def ext_slice(self, idim, start, end):
        """Index tuple selecting [start:end] along FV axis idim of an
        extended array (V, Z, Y, X)."""
        sl = [slice(None)] * (self.ndim + 1)
        sl[self.ndim - idim] = slice(start, end)
        return tuple(sl)

    def fv_boundaries(self, M, all_=True):
        """src/fv_simulator.py:224-273 on an extended array (V, ...)."""
        g = self.ngh
        for idim in range(self.ndim):
            cuts = (self.ext_slice(idim, -2 * g, -g), self.ext_slice(idim, g, 2 * g))
            for side in (0, 1):
                kind = self.BC[idim][side]
                if kind == "periodic":
                    self.BC_fv[idim][side] = M[cuts[side]]
                elif kind == "reflective":
                    if all_:
                        self.BC_fv[idim][side] = M[cuts[1 - side]]
                        self.BC_fv[idim][side][idim + 1] *= -1
                elif kind == "gradfree":
                    if all_:
                        self.BC_fv[idim][side] = M[cuts[1 - side]]
                elif kind in ("ic", "pressure"):
                    pass
                elif kind == "eq":
                    if all_:
                        self.BC_fv[idim][side][...] = 0
                else:
                    raise TypeError("Undetermined boundary type")
            M[self.ext_slice(idim, None, g)] = self.BC_fv[idim][0]
            M[self.ext_slice(idim, -g, None)] = self.BC_fv[idim][1]

    def active(self):
        g = self.ngh
        return (slice(None),) + (slice(g, -g),) * self.ndim

    def store_high_order_fluxes(self, Ffaces_t, i):
        """src/sdader_simulator.py:310-323 (time slice i) -> FV faces."""
        out = {}
        nd = self.ndim
        for idim in range(nd):
            Fi = Ffaces_t[idim][:, i]      # (V, Ncells..., pts...) SD layout
            ax_sp = sp_axis(nd, idim)
            first = _shift(Fi, None, -1, ax_sp)          # fps 0..n-1
            first_fv = self.to_fv(first)
            last = np.take(np.take(Fi, -1, axis=ax_sp), -1, axis=cell_axis(nd, idim) + 1)
            # last has shape (V, other cells..., other pts...) -> FV face row
            last_fv = self._to_fv_face(last, idim)
            out[idim] = np.concatenate(
                [first_fv, np.expand_dims(last_fv, nd - idim)], axis=nd - idim)
        return out

    def _to_fv_face(self, A, idim):
        """(V, other cells (z..x order), other pts) -> (V, other subcells)."""
        nd = self.ndim
        if nd == 1:
            return A
        if nd == 2:
            return A.reshape(A.shape[0], A.shape[1] * A.shape[2])
        return np.transpose(A, (0, 1, 3, 2, 4)).reshape(A.shape[0], A.shape[1] * A.shape[3],
                                                       A.shape[2] * A.shape[4])

    def integrate_faces(self, F_all):
        """src/sd_simulator.py:208-212."""
        out = {}
        for idim in range(self.ndim):
            M = F_all[idim]
            for od in range(self.ndim):
                if od != idim:
                    M = apply_axis(self.ops["sp_to_cv"], M, sp_axis(self.ndim, od), axis_order(od))
            out[idim] = M
        return out

    def fv_apply_fluxes(self, U_cv, F, dt):
        """src/fv_simulator.py:189-205."""
        g = self.ngh
        dUdt = None
        for idim in range(self.ndim):
            fp = self.faces[idim]
            dx = fp[g + 1:-g] - fp[g:-(g + 1)]
            dx = self.bshape(dx, idim)[np.newaxis]
            ax = self.ndim - idim
            part = (_shift(F[idim], 1, None, ax) - _shift(F[idim], None, -1, ax)) / dx
            dUdt = part if dUdt is None else dUdt + part
        return U_cv - dUdt * dt

    def detect_troubles(self, U_cv, U_new, M_fv):
        """src/trouble_detection.py:5-87; M_fv is the persistent extended array."""
        g = self.ngh
        nd = self.ndim
        W_old = compute_primitives(U_cv, nd, self.gamma)
        M_fv[self.active()] = W_old
        W_new = compute_primitives(U_new, nd, self.gamma)
        self.fv_boundaries(M_fv)
        W_max = M_fv.copy()
        W_min = M_fv.copy()
        for idim in range(nd):
            W_max = np.maximum(self._W_ex(M_fv, idim, np.maximum), W_max)
            W_min = np.minimum(self._W_ex(M_fv, idim, np.minimum), W_min)
        W_max = W_max[self.active()]
        W_min = W_min[self.active()]
        if self.p > 0:
            if self.NAD == "delta":
                eps = self.tol * (W_max - W_min)
                W_min = W_min - eps
                W_max = W_max + eps
            else:
                W_min = W_min - np.abs(W_min) * self.tol
                W_max = W_max + np.abs(W_max) * self.tol
        pt = np.where(W_new >= W_min, 0, 1)
        pt = np.where(W_new <= W_max, pt, 1)
        self.sed_ran = False
        if np.any(pt) and self.p > 1 and self.SED:
            self.sed_ran = True
            M_fv[self.active()] = W_new
            self.fv_boundaries(M_fv)
            alpha = W_new * 0 + 1
            for idim in range(nd):
                crop = [slice(None)] + [slice(g, -g)] * nd
                crop[nd - idim] = slice(None)
                alpha_new = self._smooth_extrema(M_fv, idim)[tuple(crop)]
                alpha = np.where(alpha_new < alpha, alpha_new, alpha)
            pt = pt * np.where(alpha < 1, 1, 0)
        _p_ = nd + 1
        troubles = np.maximum(pt[0], pt[_p_]).astype(np.float64)
        if self.PAD:
            troubles = np.where(W_new[0] >= self.min_rho, troubles, 1)
            troubles = np.where(W_new[0] <= self.max_rho, troubles, 1)
            troubles = np.where(W_new[_p_] >= self.min_P, troubles, 1)
        self.troubles = troubles[np.newaxis].astype(np.float64)
        M_fv[...] = 0
        M_fv[self.active()] = self.troubles
        self.fv_boundaries(M_fv, all_=False)
        trouble = M_fv[0]
        theta = trouble.copy()
        if self.blending:
            self._apply_blending(trouble, theta)
        self.theta = theta[np.newaxis]
        for idim in range(nd):
            sl1 = [slice(g, -g)] * nd
            sl2 = [slice(g, -g)] * nd
            sl1[nd - 1 - idim] = slice(g - 1, -g)
            sl2[nd - 1 - idim] = slice(g, -(g - 1))
            self.affected[idim] = np.maximum(theta[tuple(sl1)], theta[tuple(sl2)])[np.newaxis]

    def _W_ex(self, W, idim, f):
        """src/trouble_detection.py:89-102."""
        ax = self.ndim - idim
        W_f = W.copy()
        W_f[self._ax_slice(W, ax, None, -1)] = f(_shift(W, None, -1, ax), _shift(W, 1, None, ax))
        W_f[self._ax_slice(W, ax, 1, None)] = f(_shift(W_f, 1, None, ax), _shift(W_f, None, -1, ax))
        return W_f

    @staticmethod
    def _ax_slice(W, ax, start, end):
        sl = [slice(None)] * W.ndim
        sl[ax] = slice(start, end)
        return tuple(sl)

    def _smooth_extrema(self, U, idim):
        """src/trouble_detection.py:104-137 on the extended array U."""
        ax = self.ndim - idim
        cshape = [1] * U.ndim
        cshape[ax] = -1
        centers = self.centers[idim].reshape(cshape)
        hfp = self.h_fp[idim].reshape(cshape)

        def fod(A, h):
            return (_shift(A, 2, None, ax) - _shift(A, None, -2, ax)) / (_shift(h, 2, None, ax) - _shift(h, None, -2, ax))

        with np.errstate(all="ignore"):
            dU = fod(U, centers)
            d2U = fod(dU, _shift(centers, 1, -1, ax))
            dv = 0.5 * _shift(hfp, 2, -2, ax) * d2U
            vL = _shift(dU, None, -2, ax) - _shift(dU, 1, -1, ax)
            alphaL = -np.where(dv < 0, np.where(vL > 0, vL, 0), np.where(vL < 0, vL, 0)) / dv
            alphaL = np.where(np.abs(dv) <= 0, 1, alphaL)
            alphaL = np.where(alphaL < 1, alphaL, 1)
            vR = _shift(dU, 2, None, ax) - _shift(dU, 1, -1, ax)
            alphaR = np.where(dv > 0, np.where(vR > 0, vR, 0), np.where(vR < 0, vR, 0)) / dv
            alphaR = np.where(np.abs(dv) <= 0, 1, alphaR)
            alphaR = np.where(alphaR < 1, alphaR, 1)
            alphaR = np.where(alphaR < alphaL, alphaR, alphaL)
        # compute_min (src/trouble_detection.py:108-110)
        alphaL[self._ax_slice(alphaL, ax, None, -1)] = np.minimum(_shift(alphaR, None, -1, ax), _shift(alphaR, 1, None, ax))
        alphaL[self._ax_slice(alphaL, ax, 1, None)] = np.minimum(_shift(alphaR, None, -1, ax), _shift(alphaL, 1, None, ax))
        return alphaL

    def _apply_blending(self, trouble, theta):
        """src/trouble_detection.py:139-169 (in place on theta; 3D as coded)."""
        nd = self.ndim
        a = slice(None, -1)
        b = slice(1, None)

        def cut(s, idim):
            sl = [slice(None)] * nd
            sl[nd - 1 - idim] = s
            return tuple(sl)

        for idim in range(nd):
            theta[cut(a, idim)] = np.maximum(.75 * trouble[cut(b, idim)], theta[cut(a, idim)])
            theta[cut(b, idim)] = np.maximum(.75 * trouble[cut(a, idim)], theta[cut(b, idim)])
        cuts = [(a, a), (a, b), (b, a), (b, b)]
        if nd == 2:
            for i in range(4):
                theta[cuts[i]] = np.maximum(.5 * trouble[cuts[::-1][i]], theta[cuts[i]])
        elif nd == 3:
            for i in range(4):
                for idim in range(nd):
                    s1 = tuple(np.roll(np.array((slice(None),) + cuts[i], dtype=object), -idim))
                    s2 = tuple(np.roll(np.array((slice(None),) + cuts[::-1][-i], dtype=object), -idim))
                    theta[s1] = np.maximum(.5 * trouble[s2], theta[s1])
            cuts1 = [(x, y, z) for x in (a, b) for y in (a, b) for z in (a, b)]
            cuts2 = [(x, y, z) for x in (b, a) for y in (b, a) for z in (b, a)]
            for i in range(4):
                theta[cuts1[i]] = np.maximum(.375 * trouble[cuts2[i]], theta[cuts1[i]])
        for idim in range(nd):
            theta[cut(a, idim)] = np.maximum(.25 * (theta[cut(b, idim)] > 0), theta[cut(a, idim)])
            theta[cut(b, idim)] = np.maximum(.25 * (theta[cut(a, idim)] > 0), theta[cut(b, idim)])

    def muscl_hancock(self, M_fv, W_cv, dt):
        """src/fv_simulator.py:167-175 + src/muscl.py:129-221 -> F_FB per dim."""
        nd = self.ndim
        g = self.ngh
        M_fv[...] = 0
        M_fv[self.active()] = W_cv
        self.fv_boundaries(M_fv)
        S = {}
        dMhs = {}
        for idim in range(nd):
            ax = nd - idim
            hshape = [-1 if k == ax else 1 for k in range(nd + 1)]
            hcv = self.h_cv[idim].reshape(hshape)
            hfp = self.h_fp[idim].reshape(hshape)
            dMh = limited_gradient(M_fv, hcv, hfp, ax, self.limiter)
            S[idim] = 0.5 * dMh * _shift(hfp, 1, -1, ax)
            crop = [slice(None)] + [slice(1, -1)] * nd
            crop[ax] = slice(None)
            dMhs[idim] = dMh[tuple(crop)]
        inner = (slice(None),) + (slice(1, -1),) * nd
        W = M_fv[inner]
        dtW = np.zeros_like(W)
        _p_ = nd + 1
        vels = self.vels()
        for idim in range(nd):
            vel = vels[idim]
            dW = dMhs[idim]
            with np.errstate(all="ignore"):
                dtW[0] -= (W[vel] * dW[0] + W[0] * dW[vel])
                dtW[_p_] -= (W[vel] * dW[_p_] + self.gamma * W[_p_] * dW[vel])
                dtW[vel] -= (W[vel] * dW[vel] + dW[_p_] / W[0])
            for vel2 in vels[1:]:
                dtW[vel2] -= W[vel] * dW[vel2]
        dtW[_p_] *= 0
        M_fv[inner] += 0.5 * dtW * dt
        F = {}
        for idim in range(nd):
            ax = nd - idim
            crop_m = [slice(None)] + [slice(g, -g)] * nd
            crop_s = [slice(None)] + [slice(g, -g)] * nd
            crop_m[ax] = slice(g, -1)
            crop_s[ax] = slice(1, None)
            MR = M_fv[tuple(crop_m)] - S[idim][tuple(crop_s)]
            crop_m[ax] = slice(1, -g)
            crop_s[ax] = slice(None, -1)
            ML = M_fv[tuple(crop_m)] + S[idim][tuple(crop_s)]
            F[idim] = riemann(self.rs_fv, ML, MR, self.rolled_vels(idim), self.gamma,
                              self.min_c2, prims=True)
        return F

    def fv_update(self, F_all):
        """src/sdader_simulator.py:333-349 (with switch_to_* :288-307)."""
        nd = self.ndim
        U_cv = self.to_fv(apply_full(self.ops["sp_to_cv"], self.U_sp, nd))
        Ffaces = self.integrate_faces(F_all)
        g = self.ngh
        ext_shape = (self.V,) + tuple(self.N[i] * self.n + 2 * g for i in range(nd))[::-1]
        if not hasattr(self, "M_fv"):
            self.M_fv = np.zeros(ext_shape)
        w = self.ops["w_tp"]
        for i in range(self.T):
            W_cv = compute_primitives(U_cv, nd, self.gamma)
            dt = self.dt * w[i]
            F_HO = self.store_high_order_fluxes(Ffaces, i)
            U_new = self.fv_apply_fluxes(U_cv, F_HO, dt)
            if self.FB:
                self.detect_troubles(U_cv, U_new, self.M_fv)
                F_FB = self.muscl_hancock(self.M_fv, W_cv, dt)
                F = {}
                for idim in range(nd):
                    theta = 1 if self.godunov else self.affected[idim]
                    F[idim] = theta * F_FB[idim] + (1 - theta) * F_HO[idim]
                U_new = self.fv_apply_fluxes(U_cv, F, dt)
            U_cv = U_new
        self.U_cv = self.to_sd(U_cv)
        self.U_sp = apply_full(self.ops["cv_to_sp"], self.U_cv, nd, rows=True)

    # ---- drivers (src/sdader_simulator.py:361-413) -----------------------
    def perform_update(self):
        self.n_step += 1
        F_all = self.ader_predictor()
        if self.update == "SD":
            self.ader_update(F_all)
        else:
            self.fv_update(F_all)
        self.W_cv = compute_primitives(self.U_cv, self.ndim, self.gamma)
        self.time += self.dt

    def end_sim(self):
        self.U_cv = apply_full(self.ops["sp_to_cv"], self.U_sp, self.ndim)
        self.W_cv = compute_primitives(self.U_cv, self.ndim, self.gamma)

    def perform_iterations(self, n_step):
        for _ in range(n_step):
            self.compute_dt()
            self.perform_update()
        self.end_sim()

    def perform_time_evolution(self, t_end):
        while self.time < t_end:
            self.compute_dt()
            if self.time + self.dt >= t_end:
                self.dt = t_end - self.time
            if self.dt < 1e-14:
                break
            self.perform_update()
        self.end_sim()
