"""CPU oracle for the SD-ADER step of jpalafou/spd -- TEST INFRASTRUCTURE ONLY.

This module restates the reference's SD-ADER time step (predictor, SD
update, subcell finite-volume update with a-posteriori limiting) in FP64.
It exists to check the CUDA path: only ``tests/``,
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

The code never updates in place a value it has read, and every array
operation goes through the small ``xp`` dispatch below, so the same
restatement runs on NumPy arrays (the oracle proper) or on torch FP64
tensors: torch autograd through it then gives the reference gradient of the
step, with dt, the trouble masks and the blending weights detached
(frozen), as in the hand-written adjoint.

Layouts are the reference's: SD arrays are (V, [T], Nz, Ny, Nx, nz, ny, nx)
with absent dimensions dropped, FV arrays are (V, Nz*n, Ny*n, Nx*n).
"""
from __future__ import annotations

import numpy as np

try:  # torch is optional: the NumPy oracle needs none of it
    import torch
except Exception:  # pragma: no cover
    torch = None

DIMS = ("x", "y", "z")


# ----------------------------------------------------------------------------
# array-module dispatch (NumPy or torch)
# ----------------------------------------------------------------------------
def _is_t(*xs):
    return torch is not None and any(torch.is_tensor(x) for x in xs)


def _like(x, ref):
    """Python/NumPy scalar -> tensor on ref's device (torch mode)."""
    if torch.is_tensor(x):
        return x
    return torch.as_tensor(x, dtype=ref.dtype, device=ref.device)


if torch is not None:
    class _RoundedSqrt(torch.autograd.Function):
        """Correctly rounded square root (torch's CPU kernel is not) with the
        derivative 1/(2 sqrt(x))."""

        @staticmethod
        def forward(ctx, x):
            y = torch.from_numpy(np.sqrt(x.detach().cpu().numpy())).to(x.device)
            ctx.save_for_backward(y)
            return y

        @staticmethod
        def backward(ctx, g):
            (y,) = ctx.saved_tensors
            return g / (2 * y)


class xp:
    @staticmethod
    def where(c, a, b):
        if _is_t(c, a, b):
            return torch.where(c, a, b)
        return np.where(c, a, b)

    @staticmethod
    def maximum(a, b):
        if _is_t(a, b):
            ref = a if torch.is_tensor(a) else b
            return torch.maximum(_like(a, ref), _like(b, ref))
        return np.maximum(a, b)

    @staticmethod
    def minimum(a, b):
        if _is_t(a, b):
            ref = a if torch.is_tensor(a) else b
            return torch.minimum(_like(a, ref), _like(b, ref))
        return np.minimum(a, b)

    @staticmethod
    def abs(a):
        return torch.abs(a) if _is_t(a) else np.abs(a)

    @staticmethod
    def sqrt(a):
        if _is_t(a):
            return torch.sqrt(a) if a.is_cuda else _RoundedSqrt.apply(a)
        return np.sqrt(a)

    @staticmethod
    def sign(a):
        return torch.sign(a) if _is_t(a) else np.sign(a)

    @staticmethod
    def take(M, s, axis):
        if _is_t(M):
            return M.select(axis % M.dim(), s)
        return np.take(M, s, axis=axis)

    @staticmethod
    def stack(xs, axis):
        return torch.stack(xs, dim=axis) if _is_t(*xs) else np.stack(xs, axis=axis)

    @staticmethod
    def cat(xs, axis):
        return torch.cat(xs, dim=axis) if _is_t(*xs) else np.concatenate(xs, axis=axis)

    @staticmethod
    def expand(x, axis):
        return x.unsqueeze(axis) if _is_t(x) else np.expand_dims(x, axis)

    @staticmethod
    def repeat(x, n, axis):
        return x.repeat_interleave(n, dim=axis) if _is_t(x) else np.repeat(x, n, axis=axis)

    @staticmethod
    def transpose(x, perm):
        return x.permute(*perm) if _is_t(x) else np.transpose(x, perm)

    @staticmethod
    def copy(x):
        return x.clone() if _is_t(x) else np.array(x, copy=True)

    @staticmethod
    def zeros(shape, ref):
        if _is_t(ref):
            return torch.zeros(shape, dtype=torch.float64, device=ref.device)
        return np.zeros(shape)

    @staticmethod
    def f64(x):
        return x.to(torch.float64) if _is_t(x) else np.asarray(x).astype(np.float64)

    @staticmethod
    def detach(x):
        return x.detach() if _is_t(x) else x


class _Mat:
    """Operator matrix whose elements are Python floats (the same doubles,
    usable with either array module)."""

    def __init__(self, a):
        a = np.asarray(a, dtype=np.float64)
        self.shape = a.shape
        self.a = a.tolist()

    def __getitem__(self, idx):
        if isinstance(idx, tuple):
            return self.a[idx[0]][idx[1]]
        return self.a[idx]


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
    A = A if isinstance(A, _Mat) else _Mat(A)
    axis = axis % M.ndim
    n_to, n_from = A.shape
    assert M.shape[axis] == n_from
    cols = [xp.take(M, s, axis) for s in range(n_from)]
    outs = [_sum_terms([A[f, s] * cols[s] for s in range(n_from)], order) for f in range(n_to)]
    return xp.stack(outs, axis)


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
    A = A if isinstance(A, _Mat) else _Mat(A)
    n = A.shape[1]
    no = A.shape[0]
    if ndim == 1:
        return apply_axis(A, M, -1, "lanes2")
    outs = []
    if ndim == 2:
        for j in range(no):
            for i in range(no):
                if rows or n == 2:
                    row_sums = [_sum_terms([(A[j, m] * A[i, l]) * M[..., m, l] for l in range(n)], "seq")
                                for m in range(n)]
                    outs.append(_sum_terms(row_sums, "seq"))
                else:
                    outs.append(_sum_terms([(A[j, m] * A[i, l]) * M[..., m, l]
                                            for m in range(n) for l in range(n)], "seq"))
        return xp.stack(outs, -1).reshape(tuple(M.shape[:-2]) + (no, no))
    for k in range(no):
        for j in range(no):
            for i in range(no):
                if rows:
                    row_sums = [_sum_terms([((A[k, a] * A[j, b]) * A[i, c]) * M[..., a, b, c] for c in range(n)],
                                           "seq")
                                for a in range(n) for b in range(n)]
                    outs.append(_sum_terms(row_sums, "seq"))
                else:
                    outs.append(_sum_terms([((A[k, a] * A[j, b]) * A[i, c]) * M[..., a, b, c]
                                            for a in range(n) for b in range(n) for c in range(n)], "seq"))
    return xp.stack(outs, -1).reshape(tuple(M.shape[:-3]) + (no, no, no))


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
def compute_primitives(U, ndim, gamma, vels=None, iso=False):
    """src/hydro.py:48-86 (U -> W); the kinetic term sums in ``vels`` order;
    ``iso``: the isothermal system multiplies the kinetic term by 0."""
    _p_ = ndim + 1
    comp = {0: U[0]}
    K = None
    for vel in (range(1, ndim + 1) if vels is None else vels):
        comp[vel] = U[vel] / U[0]
        K = comp[vel] * comp[vel] if K is None else K + comp[vel] * comp[vel]
    K = K * (0.5 * U[0])
    if iso:
        K = K * 0
    comp[_p_] = (gamma - 1) * (U[_p_] - K)
    return xp.stack([comp[v] for v in range(ndim + 2)], 0)


def compute_conservatives(W, ndim, gamma, vels=None, iso=False):
    """src/hydro.py:88-125 (W -> U); the kinetic term sums in ``vels`` order."""
    _p_ = ndim + 1
    comp = {0: W[0]}
    K = None
    for vel in (range(1, ndim + 1) if vels is None else vels):
        comp[vel] = W[vel] * W[0]
        K = W[vel] * W[vel] if K is None else K + W[vel] * W[vel]
    K = K * (0.5 * W[0])
    if iso:
        K = K * 0
    comp[_p_] = W[_p_] / (gamma - 1) + K
    return xp.stack([comp[v] for v in range(ndim + 2)], 0)


def compute_fluxes(W, vels, gamma, iso=False):
    """src/hydro.py:127-170; ``vels`` is the rotated velocity index list;
    the isothermal system multiplies the energy flux by 0."""
    ndim = len(vels)
    _p_ = ndim + 1
    comp = {}
    v1 = vels[0]
    K = None
    m = None
    for v in vels[::-1]:
        m = W[0] * W[v]
        K = m * W[v] if K is None else K + m * W[v]
        comp[v] = m * W[v1]
    E = W[_p_] / (gamma - 1) + 0.5 * K
    comp[0] = m
    comp[v1] = m * W[v1] + W[_p_]
    comp[_p_] = W[v1] * (E + W[_p_])
    if iso:
        comp[_p_] = comp[_p_] * 0
    return xp.stack([comp[v] for v in range(ndim + 2)], 0)


def viscous_fluxes(W, vels, dUs, nu, beta):
    """src/hydro.py:172-241: viscous fluxes of the conservative variables
    from the primitives W and their gradients dUs[direction], in the
    rotated velocity order ``vels``; the density component is 0*rho*nu."""
    ndim = len(vels)
    _p_ = ndim + 1
    v1 = vels[0]
    dU1 = dUs[v1 - 1]
    comp = {}
    comp[v1] = 2 * dU1[v1] - beta * dU1[v1]
    comp[_p_] = W[v1] * comp[v1]
    for vel in vels[1:]:
        dU = dUs[vel - 1]
        comp[v1] = comp[v1] - beta * dU[vel]
        comp[vel] = dU1[vel] + dU[v1]
        comp[_p_] = comp[_p_] + W[vel] * comp[vel]
    return xp.stack([(comp[v] if v else xp.zeros(W[0].shape, W)) * W[0] * nu for v in range(ndim + 2)], 0)


def compute_cs(P, rho, gamma, min_c2):
    """src/hydro.py:3-46: sqrt of gamma*P/rho floored at min_c2 (NaN -> floor)."""
    c2 = gamma * P / rho
    c2 = xp.where(c2 > min_c2, c2, min_c2)
    return xp.sqrt(c2)


# ----------------------------------------------------------------------------
# Riemann solvers (src/riemann_solver.py)
# ----------------------------------------------------------------------------
def riemann(name, M_L, M_R, vels, gamma, min_c2, prims, iso=False):
    """src/riemann_solver.py:10-29 wrapper, then llf/hllc/lhllc."""
    ndim = len(vels)
    if prims:
        W_L, W_R = M_L, M_R
        U_L = compute_conservatives(W_L, ndim, gamma, vels, iso)
        U_R = compute_conservatives(W_R, ndim, gamma, vels, iso)
    else:
        U_L, U_R = M_L, M_R
        W_L = compute_primitives(U_L, ndim, gamma, vels, iso)
        W_R = compute_primitives(U_R, ndim, gamma, vels, iso)
    if name == "llf":
        return _llf(W_L, W_R, U_L, U_R, vels, gamma, min_c2, iso)
    if name in ("hllc", "lhllc"):
        return _hllc(W_L, W_R, U_L, U_R, vels, gamma, min_c2, low_mach=(name == "lhllc"), iso=iso)
    raise AttributeError(name)


def _llf(W_L, W_R, U_L, U_R, vels, gamma, min_c2, iso=False):
    """src/riemann_solver.py:31-65."""
    _p_ = len(vels) + 1
    v1 = vels[0]
    F_L = compute_fluxes(W_L, vels, gamma, iso)
    F_R = compute_fluxes(W_R, vels, gamma, iso)
    c_L = compute_cs(W_L[_p_], W_L[0], gamma, min_c2) + xp.abs(W_L[v1])
    c_R = compute_cs(W_R[_p_], W_R[0], gamma, min_c2) + xp.abs(W_R[v1])
    c_max = xp.where(c_L > c_R, c_L, c_R)[None, ...]
    return 0.5 * (F_R + F_L) - 0.5 * c_max * (U_R - U_L)


def _hllc(W_L, W_R, U_L, U_R, vels, gamma, min_c2, low_mach=False, iso=False):
    """src/riemann_solver.py:67-145 (hllc) and :147-212 (lhllc)."""
    _p_ = len(vels) + 1
    v1 = vels[0]
    c_L = compute_cs(W_L[_p_], W_L[0], gamma, min_c2) + xp.abs(W_L[v1])
    c_R = compute_cs(W_R[_p_], W_R[0], gamma, min_c2) + xp.abs(W_R[v1])
    c_max = xp.where(c_L > c_R, c_L, c_R)
    v_L = W_L[v1]
    v_R = W_R[v1]
    s_L = xp.where(v_L < v_R, v_L, v_R) - c_max
    s_R = xp.where(v_L > v_R, v_L, v_R) + c_max
    rc_L = W_L[0] * (v_L - s_L)
    rc_R = W_R[0] * (s_R - v_R)
    with np.errstate(all="ignore"):
        v_star = (rc_R * v_R + rc_L * v_L + (W_L[_p_] - W_R[_p_])) / (rc_R + rc_L)
        if low_mach:
            Mach = xp.minimum(1.0, xp.maximum(xp.abs(v_L), xp.abs(v_R)) / c_max)
            phi = Mach * (2 - Mach)
            P_star = (rc_R * W_L[_p_] + rc_L * W_R[_p_] + phi * rc_L * rc_R * (v_L - v_R)) / (rc_R + rc_L)
        else:
            P_star = (rc_R * W_L[_p_] + rc_L * W_R[_p_] + rc_L * rc_R * (v_L - v_R)) / (rc_R + rc_L)
        r_starL = W_L[0] * (s_L - v_L) / (s_L - v_star)
        e_starL = ((s_L - v_L) * U_L[_p_] - W_L[_p_] * v_L + P_star * v_star) / (s_L - v_star)
        r_starR = W_R[0] * (s_R - v_R) / (s_R - v_star)
        e_starR = ((s_R - v_R) * U_R[_p_] - W_R[_p_] * v_R + P_star * v_star) / (s_R - v_star)
    r_gdv = xp.where(s_L > 0, W_L[0], xp.where(v_star > 0, r_starL, xp.where(s_R > 0, r_starR, W_R[0])))
    v_gdv = xp.where(s_L > 0, v_L, xp.where(v_star > 0, v_star, xp.where(s_R > 0, v_star, v_R)))
    P_gdv = xp.where(s_L > 0, W_L[_p_], xp.where(v_star > 0, P_star, xp.where(s_R > 0, P_star, W_R[_p_])))
    e_gdv = xp.where(s_L > 0, U_L[_p_], xp.where(v_star > 0, e_starL, xp.where(s_R > 0, e_starR, U_R[_p_])))
    comp = {0: r_gdv * v_gdv}
    comp[v1] = comp[0] * v_gdv + P_gdv
    comp[_p_] = v_gdv * (e_gdv + P_gdv)
    for vel in vels[1:]:
        comp[vel] = comp[0] * xp.where(v_star > 0, W_L[vel], W_R[vel])
    if iso:
        comp[_p_] = comp[_p_] * 0
    return xp.stack([comp[v] for v in range(len(vels) + 2)], 0)


# ----------------------------------------------------------------------------
# slope limiters and MUSCL-Hancock (src/muscl.py)
# ----------------------------------------------------------------------------
def _shift(M, start, end, axis):
    sl = [slice(None)] * M.ndim
    sl[axis] = slice(start, end)
    return M[tuple(sl)]


def minmod_branch(SL, SR):
    """Branch of the reference's minmod (src/muscl.py:33-35) taken at each
    point: 0 -> 0*SL (ratio <= 0), 1 -> ratio*SL (0 < ratio < 1), 2 -> SL
    (ratio >= 1 or NaN, which includes SL = 0)."""
    SL = xp.detach(SL)
    SR = xp.detach(SR)
    with np.errstate(all="ignore"):
        r = SR / SL
    lt1 = r < 1
    return xp.where(lt1 & (r > 0), 1, xp.where(lt1, 0, 2))


def minmod(SL, SR, branch=None):
    """src/muscl.py:12-35 (ratio form; NaN ratio -> SL).  Evaluated branch by
    branch so that the torch form keeps NaN out of the gradient; ``branch``
    (from minmod_branch) replays a recorded choice."""
    if branch is None:
        branch = minmod_branch(SL, SR)
    with np.errstate(all="ignore"):
        safe = xp.where((branch == 1) & (SL != 0), SL, 1.0)
        mid = (SR / safe) * SL
    return xp.where(branch == 1, mid, xp.where(branch == 2, SL, 0 * SL))


def moncen(dU_L, dU_R, dx_L, dx_R, dx_M):
    """src/muscl.py:37-59."""
    dU_C = (dx_L * dU_L + dx_R * dU_R) / (dx_L + dx_R)
    slope = xp.minimum(xp.abs(2 * dU_L * dx_L / dx_M), xp.abs(2 * dU_R * dx_R / dx_M))
    slope = xp.sign(dU_C) * xp.minimum(slope, xp.abs(dU_C))
    return xp.where(dU_L * dU_R >= 0, slope, 0.0)


def limited_gradient(M, h_cv, h_fp, axis, limiter, branch=None, record=None):
    """src/muscl.py:61-75 along array axis ``axis`` (h arrays broadcast)."""
    dM = (_shift(M, 1, None, axis) - _shift(M, None, -1, axis)) / h_cv
    SL = _shift(dM, None, -1, axis)
    SR = _shift(dM, 1, None, axis)
    if limiter == "minmod":
        if branch is None:
            branch = minmod_branch(SL, SR)
        if record is not None:
            record.append(branch)
        return minmod(SL, SR, branch)
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


def _whole_axis(idx, ax):
    """An index tuple with axis ``ax`` left whole."""
    sl = list(idx)
    sl[ax] = slice(None)
    return tuple(sl)


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
    NumPy arrays run the oracle; torch FP64 tensors run the same
    restatement under autograd.
    """

    def __init__(self, *, ndim, N, p, m, lims, BC, gamma, cfl_coeff, min_c2,
                 riemann_solver_sd, riemann_solver_fv, slope_limiter, update,
                 FB, tolerance, SED, NAD, PAD, blending, min_rho, max_rho,
                 min_P, godunov, ops, state, Nghc=2, viscosity=False, nu=1e-4, beta=2.0 / 3, potential=False,
                 isothermal=False, WB=False):
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
        self.viscosity = viscosity
        self.nu = nu
        self.beta = beta
        self.potential = potential
        self.iso = isothermal
        self.ngh = Nghc
        self.ops = {k: (_Mat(v) if k in ("sp_to_fp", "dfp_to_sp", "sp_to_cv", "cv_to_sp", "invader", "w_tp")
                        else v) for k, v in ops.items()}
        self.h = [(lims[i][1] - lims[i][0]) / self.N[i] for i in range(ndim)]
        self.h_min = 1e10
        for hh in self.h:
            self.h_min = min(self.h_min, hh)
        ref = state["U_sp"]
        self.torch_mode = _is_t(ref)

        def conv(a):
            if self.torch_mode and not torch.is_tensor(a):
                return torch.as_tensor(np.array(a, dtype=np.float64), device=ref.device)
            return a if self.torch_mode else np.array(a, dtype=np.float64, copy=True)

        self.U_sp = conv(state["U_sp"])
        self.U_cv = conv(state["U_cv"])
        self.W_cv = conv(state["W_cv"])
        # gravity potential gradients (src/sdader_simulator.py:425-434): at
        # the solution points (ndim, cells..., points...) and as subcell
        # averages in the FV layout (ndim, subcells...)
        if potential:
            self.grad_phi_sp = conv(state["grad_phi_sp"])
            self.grad_phi_fv = conv(state["grad_phi_fv"])
        # well-balanced mode (src/sdader_simulator.py:436-481): the step
        # advances the perturbation U - U_eq; equilibrium states at the
        # solution points (U_eq_sp), as subcell averages (U_eq_cv, SD
        # layout), at the flux points of each direction with matched
        # element-interface values (M_eq_fp, conservative) and their fluxes
        # (F_eq_fp); with the FV update the primitive equilibrium at the
        # subcell faces (M_eq_faces) with its fluxes and on the extended
        # subcell grid (M_eq_fv)
        self.WB = WB
        if WB:
            self.U_eq_sp = conv(state["U_eq_sp"])
            self.U_eq_cv = conv(state["U_eq_cv"])
            self.M_eq_fp = {i: conv(state[f"M_eq_fp_{DIMS[i]}"]) for i in range(ndim)}
            self.F_eq_fp = {i: conv(state[f"F_eq_fp_{DIMS[i]}"]) for i in range(ndim)}
            if update == "FV":
                self.M_eq_faces = {i: conv(state[f"M_eq_faces_{DIMS[i]}"]) for i in range(ndim)}
                self.F_eq_faces = {i: conv(state[f"F_eq_faces_{DIMS[i]}"]) for i in range(ndim)}
                self.M_eq_fv = conv(state["M_eq_fv"])
        self.BC_fp = {i: conv(state[f"BC_fp_{DIMS[i]}"]) for i in range(ndim) if f"BC_fp_{DIMS[i]}" in state}
        self.BC_fv = {}
        for i in range(ndim):
            key = f"BC_fv_{DIMS[i]}"
            if key in state:
                b = conv(state[key])
                self.BC_fv[i] = [b[0], b[1]]
        self.time = 0.0
        self.n_step = 0
        self.dt = None
        # subcell geometry (src/sdader_simulator.py:61-92)
        self.faces, self.centers, self.h_fp, self.h_cv = [], [], [], []
        for i in range(ndim):
            fp = subcell_faces(self.N[i], self.h[i], np.asarray(ops["x_fp"]), self.ngh)
            cv = 0.5 * (fp[1:] + fp[:-1])
            self.faces.append(conv(fp))
            self.centers.append(conv(cv))
            self.h_fp.append(conv(fp[1:] - fp[:-1]))
            self.h_cv.append(conv(cv[1:] - cv[:-1]))
        self.troubles = None
        self.theta = None
        self.affected = {}
        # frozen-mask replay: when ``replay_affected`` is a list, substep k
        # of the run uses its k-th entry as the affected faces instead of
        # detecting troubles (for finite differences of the frozen-mask map)
        self.replay_affected = None
        self.record_affected = []
        self.replay_minmod = None
        self.record_minmod = []

    # ---- helpers --------------------------------------------------------
    def vels(self):
        return list(range(1, self.ndim + 1))

    def rolled_vels(self, idim):
        return [int(v) for v in np.roll(np.arange(1, self.ndim + 1), -idim)]

    def line(self, arr, idim, nd):
        """1D array along FV axis idim, broadcast over an nd-axis array."""
        shp = [1] * nd
        shp[nd - 1 - idim] = -1
        return arr.reshape(shp)

    # ---- dt (src/sd_simulator.py:214-227) --------------------------------
    def compute_dt(self):
        """The CFL step, a Python float (detached from any graph)."""
        W = xp.detach(self.W_cv)
        _p_ = self.ndim + 1
        c_s = compute_cs(W[_p_], W[0], self.gamma, self.min_c2)
        c = c_s * self.ndim
        for vel in self.vels():
            c = c + xp.abs(W[vel])
        c_max = float(c.max())
        h = self.h_min / (self.p + 1)
        dt = h / c_max if c_max == c_max else float("nan")
        if self.viscosity and self.nu > 0:
            # Python's min keeps its first argument unless the second is smaller
            dt = min(dt, h ** 2 / self.nu * .25)
        self.dt = self.cfl * dt
        return self.dt

    # ---- predictor (src/sdader_simulator.py:160-240) ---------------------
    def solve_faces(self, U_ader):
        """Returns F_ader_fp per dim with Riemann fluxes at element edges."""
        ops = self.ops
        nd = self.ndim
        F_all, M_all = {}, {}
        for idim in range(nd):
            vels = self.rolled_vels(idim)
            ax_sp = sp_axis(nd, idim)
            ax_cell = cell_axis(nd, idim)
            M_fp = apply_axis(ops["sp_to_fp"], U_ader, ax_sp, axis_order(idim))
            if self.WB:
                # U' -> U at the flux points (src/sdader_simulator.py:221-223)
                M_fp = M_fp + xp.expand(self.M_eq_fp[idim], 1)
            # interior flux points (the edge values are replaced below)
            M_in = _shift(M_fp, 1, -1, ax_sp)
            F_in = compute_fluxes(compute_primitives(M_in, nd, self.gamma, iso=self.iso), vels, self.gamma, self.iso)
            ML, MR = self._interfaces(M_fp, idim)
            F = riemann(self.rs_sd, ML, MR, vels, self.gamma, self.min_c2, prims=False, iso=self.iso)
            F_all[idim] = xp.cat([xp.expand(_shift(F, None, -1, ax_cell + 1), ax_sp), F_in,
                                  xp.expand(_shift(F, 1, None, ax_cell + 1), ax_sp)], ax_sp)
            if self.WB:
                # F -> F' (src/sdader_simulator.py:235-237)
                F_all[idim] = F_all[idim] - xp.expand(self.F_eq_fp[idim], 1)
            M_all[idim] = M_fp
        if self.viscosity:
            F_all = self.add_viscosity(M_all, F_all)
        return F_all

    def _interfaces(self, M_fp, idim):
        """The left and right states at the element interfaces along idim of
        a flux-point array M_fp (the sp axis of idim holds the nf points):
        src/sd_boundary.py:70-76 (store_BC, store_interfaces, apply_BC),
        including a "pressure" side's overwrite of the domain-edge state by
        its stored boundary state."""
        nd = self.ndim
        ax_sp = sp_axis(nd, idim)
        tax = cell_axis(nd, idim) + 1
        left_trace = xp.take(M_fp, 0, ax_sp)
        right_trace = xp.take(M_fp, self.nf - 1, ax_sp)
        Ncell = self.N[idim]
        first_l = xp.take(left_trace, 0, tax)
        last_r = xp.take(right_trace, Ncell - 1, tax)
        bc = []
        for side in (0, 1):
            kind = self.BC[idim][side]
            if kind == "periodic":
                v = last_r if side == 0 else first_l
            elif kind in ("reflective", "gradfree"):
                v = first_l if side == 0 else last_r
                if kind == "reflective":
                    v = xp.stack([v[k] * -1 if k == idim + 1 else v[k] for k in range(self.V)], 0)
            elif kind in ("ic", "eq", "pressure"):
                b = self.BC_fp[idim][side]
                v = (b.expand(first_l.shape) if self.torch_mode
                     else np.broadcast_to(b, first_l.shape).copy())
            else:
                raise TypeError("Undetermined boundary type")
            bc.append(v)
        # pressure sides overwrite the edge traces with the stored state
        if self.BC[idim][0] == "pressure":
            left_trace = xp.cat([xp.expand(bc[0], tax), _shift(left_trace, 1, None, tax)], tax)
        if self.BC[idim][1] == "pressure":
            right_trace = xp.cat([_shift(right_trace, None, -1, tax), xp.expand(bc[1], tax)], tax)
        ML = xp.cat([xp.expand(bc[0], tax), right_trace], tax)
        MR = xp.cat([left_trace, xp.expand(bc[1], tax)], tax)
        return ML, MR

    def _apply_interfaces(self, X, M_fp, idim):
        """src/sd_boundary.py:19-30: interface values X into the two edge
        flux points of every cell (edge 0 of cell i <- X[i], edge nf-1 <-
        X[i+1])."""
        nd = self.ndim
        ax_sp = sp_axis(nd, idim)
        tax = cell_axis(nd, idim) + 1
        return xp.cat([xp.expand(_shift(X, None, -1, tax), ax_sp), _shift(M_fp, 1, -1, ax_sp),
                       xp.expand(_shift(X, 1, None, tax), ax_sp)], ax_sp)

    def add_viscosity(self, M_all, F_all):
        """src/sdader_simulator.py:245-268 with src/hydro.py:172-241: the
        viscous flux subtracted at every flux point.  Primitives at the flux
        points take the left state at element interfaces (ML); their
        gradient at the solution points, interpolated to the flux points of
        each direction, takes the right state (MR)."""
        nd = self.ndim
        W_fp, dW_sp = {}, {}
        for idim in range(nd):
            Wf = compute_primitives(M_all[idim], nd, self.gamma, iso=self.iso)
            ML, _ = self._interfaces(Wf, idim)
            W_fp[idim] = self._apply_interfaces(ML, Wf, idim)
            dW_sp[idim] = apply_axis(self.ops["dfp_to_sp"], W_fp[idim], sp_axis(nd, idim),
                                     axis_order(idim)) / self.h[idim]
        out = {}
        for idim in range(nd):
            vels = self.rolled_vels(idim)
            dW_fp = {}
            for e in range(nd):
                G = apply_axis(self.ops["sp_to_fp"], dW_sp[e], sp_axis(nd, idim), axis_order(idim))
                _, MR = self._interfaces(G, idim)
                dW_fp[e] = self._apply_interfaces(MR, G, idim)
            out[idim] = F_all[idim] - viscous_fluxes(W_fp[idim], vels, dW_fp, self.nu, self.beta)
        return out

    def ader_dudt(self, F_all, U_ader):
        """src/sdader_simulator.py:148-158 with src/sd_simulator.py:196-206."""
        dUdt = None
        for idim in range(self.ndim):
            part = apply_axis(self.ops["dfp_to_sp"], F_all[idim], sp_axis(self.ndim, idim),
                              axis_order(idim)) / self.h[idim]
            dUdt = part if dUdt is None else dUdt + part
        if self.potential:
            dUdt = self.apply_potential(dUdt, U_ader, xp.expand(self.grad_phi_sp, 1))
        return dUdt

    def apply_potential(self, dUdt, U, grad_phi):
        """src/simulator.py:197-203: the gravity source, dUdt[vel] += rho *
        dphi/dx_vel and dUdt[P] += m_vel * dphi/dx_vel, direction by
        direction."""
        comp = [dUdt[v] for v in range(self.V)]
        _p_ = self.ndim + 1
        for idim in range(self.ndim):
            vel = idim + 1
            comp[vel] = comp[vel] + U[0] * grad_phi[idim]
            if not self.iso:
                comp[_p_] = comp[_p_] + U[vel] * grad_phi[idim]
        return xp.stack(comp, 0)

    def ader_predictor(self):
        """src/sdader_simulator.py:160-200; returns the last F_ader_fp."""
        T = self.T
        U_ader = xp.repeat(self.U_sp[:, None], T, 1)
        inv = self.ops["invader"]
        F_all = None
        for it in range(self.m + 1):
            F_all = self.solve_faces(U_ader)
            self.U_ader = U_ader
            if it < self.m:
                dudt = self.ader_dudt(F_all, U_ader)
                cols = [dudt[:, pp] for pp in range(T)]
                terms_n = [_sum_terms([inv[nn, pp] * cols[pp] for pp in range(T)], "seq") for nn in range(T)]
                upd = xp.stack(terms_n, 1) * self.dt
                U_ader = self.U_sp[:, None] - upd
        self.F_ader = F_all
        return F_all

    def ader_update(self, F_all):
        """src/sdader_simulator.py:202-208."""
        dudt = self.ader_dudt(F_all, self.U_ader)
        w = self.ops["w_tp"]
        dUdt = _sum_terms([w[t] * dudt[:, t] for t in range(self.T)], "seq") * self.dt
        self.U_sp = self.U_sp - dUdt

    # ---- SD <-> FV layouts (src/sd_simulator.py:104-131) -----------------
    def to_fv(self, M):
        nd = self.ndim
        if nd == 1:
            return M.reshape(M.shape[0], M.shape[1] * M.shape[2])
        if nd == 2:
            return xp.transpose(M, (0, 1, 3, 2, 4)).reshape(
                M.shape[0], M.shape[1] * M.shape[3], M.shape[2] * M.shape[4])
        return xp.transpose(M, (0, 1, 4, 2, 5, 3, 6)).reshape(
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
            return xp.transpose(M.reshape(shape), (0, 1, 3, 2, 4))
        return xp.transpose(M.reshape(shape), (0, 1, 3, 5, 2, 4, 6))

    # ---- FV machinery (src/fv_simulator.py, src/trouble_detection.py) ----
    def ext_slice(self, idim, start, end):
        """Index tuple selecting [start:end] along FV axis idim of an
        extended array (V, Z, Y, X)."""
        sl = [slice(None)] * (self.ndim + 1)
        sl[self.ndim - idim] = slice(start, end)
        return tuple(sl)

    def pad(self, A):
        """Active-region array (V, ...) -> extended array with zero ghosts."""
        g = self.ngh
        out = A
        for idim in range(self.ndim):
            ax = self.ndim - idim
            zshape = list(out.shape)
            zshape[ax] = g
            z = xp.zeros(tuple(zshape), A)
            out = xp.cat([z, out, z], ax)
        return out

    def fv_boundaries(self, M, all_=True):
        """src/fv_simulator.py:224-273 on an extended array (V, ...): returns
        the filled array and updates the persistent boundary buffers (stale
        for reflective/gradfree sides when all_ is False, as in the
        reference)."""
        g = self.ngh
        for idim in range(self.ndim):
            ax = self.ndim - idim
            cuts = (self.ext_slice(idim, -2 * g, -g), self.ext_slice(idim, g, 2 * g))
            for side in (0, 1):
                kind = self.BC[idim][side]
                if kind == "periodic":
                    self.BC_fv[idim][side] = M[cuts[side]]
                elif kind in ("reflective", "gradfree"):
                    if all_:
                        src = M[cuts[1 - side]]
                        if kind == "reflective":
                            src = xp.stack([src[k] * -1 if k == idim + 1 else src[k]
                                            for k in range(src.shape[0])], 0)
                        self.BC_fv[idim][side] = src
                elif kind in ("ic", "pressure"):
                    pass
                elif kind == "eq":
                    if all_:
                        self.BC_fv[idim][side] = self.BC_fv[idim][side] * 0
                else:
                    raise TypeError("Undetermined boundary type")
            M = xp.cat([self.BC_fv[idim][0][:M.shape[0]], _shift(M, g, -g, ax),
                        self.BC_fv[idim][1][:M.shape[0]]], ax)
        return M

    def store_high_order_fluxes(self, Ffaces_t, i):
        """src/sdader_simulator.py:310-323 (time slice i) -> FV faces."""
        out = {}
        nd = self.ndim
        for idim in range(nd):
            Fi = Ffaces_t[idim][:, i]      # (V, Ncells..., pts...) SD layout
            ax_sp = sp_axis(nd, idim)
            first_fv = self.to_fv(_shift(Fi, None, -1, ax_sp))          # fps 0..n-1
            last = xp.take(xp.take(Fi, self.nf - 1, ax_sp), self.N[idim] - 1, cell_axis(nd, idim) + 1)
            last_fv = self._to_fv_face(last, idim)
            out[idim] = xp.cat([first_fv, xp.expand(last_fv, nd - idim)], nd - idim)
        return out

    def _to_fv_face(self, A, idim):
        """(V, other cells (z..x order), other pts) -> (V, other subcells)."""
        nd = self.ndim
        if nd == 1:
            return A
        if nd == 2:
            return A.reshape(A.shape[0], A.shape[1] * A.shape[2])
        return xp.transpose(A, (0, 1, 3, 2, 4)).reshape(A.shape[0], A.shape[1] * A.shape[3],
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
            dx = self.line(dx, idim, self.ndim)[None]
            ax = self.ndim - idim
            part = (_shift(F[idim], 1, None, ax) - _shift(F[idim], None, -1, ax)) / dx
            dUdt = part if dUdt is None else dUdt + part
        if self.potential:
            dUdt = self.apply_potential(dUdt, U_cv, self.grad_phi_fv)
        return U_cv - dUdt * dt

    def detect_troubles(self, U_cv, U_new):
        """src/trouble_detection.py:5-87.  Sets troubles, theta and the
        affected faces (detached: frozen in the adjoint).  The reference
        writes W_old into the active region of a persistent array whose
        ghosts its boundary fill then overwrites entirely, so the array is
        rebuilt here from the active values."""
        g = self.ngh
        nd = self.ndim
        U_cv = xp.detach(U_cv)
        U_new = xp.detach(U_new)
        W_old = self.prims_cv(U_cv)
        W_new = self.prims_cv(U_new)
        M = self.fv_boundaries(self.pad(W_old))
        act = (slice(None),) + (slice(g, -g),) * nd
        center = M[act]
        W_max = center
        W_min = center
        for idim in range(nd):
            ax = nd - idim
            lo = _shift(M, g - 1, -g - 1, ax)[_whole_axis(act, ax)]
            hi = _shift(M, g + 1, -g + 1, ax)[_whole_axis(act, ax)]
            W_max = xp.maximum(xp.maximum(xp.maximum(lo, center), hi), W_max)
            W_min = xp.minimum(xp.minimum(xp.minimum(lo, center), hi), W_min)
        if self.p > 0:
            if self.NAD == "delta":
                eps = self.tol * (W_max - W_min)
                W_min = W_min - eps
                W_max = W_max + eps
            else:
                W_min = W_min - xp.abs(W_min) * self.tol
                W_max = W_max + xp.abs(W_max) * self.tol
        pt = xp.where(W_new >= W_min, 0, 1)
        pt = xp.where(W_new <= W_max, pt, 1)
        if bool(pt.any()) and self.p > 1 and self.SED:
            Mn = self.fv_boundaries(self.pad(W_new))
            alpha = W_new * 0 + 1
            for idim in range(nd):
                crop = [slice(None)] + [slice(g, -g)] * nd
                crop[nd - idim] = slice(None)
                alpha_new = self._smooth_extrema(Mn, idim)[tuple(crop)]
                alpha = xp.where(alpha_new < alpha, alpha_new, alpha)
            pt = pt * xp.where(alpha < 1, 1, 0)
        _p_ = nd + 1
        troubles = xp.f64(xp.maximum(pt[0], pt[_p_]))
        if self.PAD:
            if self.WB:
                W_new = W_new + compute_primitives(self.to_fv(self.U_eq_cv), nd, self.gamma, iso=self.iso)
            troubles = xp.where(W_new[0] >= self.min_rho, troubles, 1.0)
            troubles = xp.where(W_new[0] <= self.max_rho, troubles, 1.0)
            troubles = xp.where(W_new[_p_] >= self.min_P, troubles, 1.0)
        self.troubles = xp.f64(troubles[None])
        tr = self.pad(xp.repeat(self.troubles, self.V, 0))
        trouble = self.fv_boundaries(tr, all_=False)[0]
        theta = self._apply_blending(trouble) if self.blending else xp.copy(trouble)
        self.theta = theta[None]
        for idim in range(nd):
            sl1 = [slice(g, -g)] * nd
            sl2 = [slice(g, -g)] * nd
            sl1[nd - 1 - idim] = slice(g - 1, -g)
            sl2[nd - 1 - idim] = slice(g, -(g - 1))
            self.affected[idim] = xp.maximum(theta[tuple(sl1)], theta[tuple(sl2)])[None]

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
            alphaL = -xp.where(dv < 0, xp.where(vL > 0, vL, 0.0), xp.where(vL < 0, vL, 0.0)) / dv
            alphaL = xp.where(xp.abs(dv) <= 0, 1.0, alphaL)
            alphaL = xp.where(alphaL < 1, alphaL, 1.0)
            vR = _shift(dU, 2, None, ax) - _shift(dU, 1, -1, ax)
            alphaR = xp.where(dv > 0, xp.where(vR > 0, vR, 0.0), xp.where(vR < 0, vR, 0.0)) / dv
            alphaR = xp.where(xp.abs(dv) <= 0, 1.0, alphaR)
            alphaR = xp.where(alphaR < 1, alphaR, 1.0)
            alphaR = xp.where(alphaR < alphaL, alphaR, alphaL)
        # compute_min (src/trouble_detection.py:108-110): a first sweep, then
        # a second one over the updated values
        first = xp.cat([xp.minimum(_shift(alphaR, None, -1, ax), _shift(alphaR, 1, None, ax)),
                        _shift(alphaL, -1, None, ax)], ax)
        return xp.cat([_shift(first, None, 1, ax),
                       xp.minimum(_shift(alphaR, None, -1, ax), _shift(first, 1, None, ax))], ax)

    def _apply_blending(self, trouble):
        """src/trouble_detection.py:139-169 (3D as coded); returns theta
        (values only: the masks carry no gradient)."""
        theta = xp.copy(trouble)
        nd = self.ndim
        a = slice(None, -1)
        b = slice(1, None)

        def cut(s, idim):
            sl = [slice(None)] * nd
            sl[nd - 1 - idim] = s
            return tuple(sl)

        for idim in range(nd):
            theta[cut(a, idim)] = xp.maximum(.75 * trouble[cut(b, idim)], theta[cut(a, idim)])
            theta[cut(b, idim)] = xp.maximum(.75 * trouble[cut(a, idim)], theta[cut(b, idim)])
        cuts = [(a, a), (a, b), (b, a), (b, b)]
        if nd == 2:
            for i in range(4):
                theta[cuts[i]] = xp.maximum(.5 * trouble[cuts[::-1][i]], theta[cuts[i]])
        elif nd == 3:
            for i in range(4):
                for idim in range(nd):
                    s1 = tuple(np.roll(np.array((slice(None),) + cuts[i], dtype=object), -idim))
                    s2 = tuple(np.roll(np.array((slice(None),) + cuts[::-1][-i], dtype=object), -idim))
                    theta[s1] = xp.maximum(.5 * trouble[s2], theta[s1])
            cuts1 = [(x, y, z) for x in (a, b) for y in (a, b) for z in (a, b)]
            cuts2 = [(x, y, z) for x in (b, a) for y in (b, a) for z in (b, a)]
            for i in range(4):
                theta[cuts1[i]] = xp.maximum(.375 * trouble[cuts2[i]], theta[cuts1[i]])
        for idim in range(nd):
            theta[cut(a, idim)] = xp.maximum(.25 * xp.f64(theta[cut(b, idim)] > 0), theta[cut(a, idim)])
            theta[cut(b, idim)] = xp.maximum(.25 * xp.f64(theta[cut(a, idim)] > 0), theta[cut(b, idim)])
        return theta

    def muscl_hancock(self, W_cv, dt):
        """src/fv_simulator.py:167-175 + src/muscl.py:129-221 -> F_FB per dim."""
        nd = self.ndim
        g = self.ngh
        M = self.fv_boundaries(self.pad(W_cv))
        S = {}
        dMhs = {}
        for idim in range(nd):
            ax = nd - idim
            hshape = [-1 if k == ax else 1 for k in range(nd + 1)]
            hcv = self.h_cv[idim].reshape(hshape)
            hfp = self.h_fp[idim].reshape(hshape)
            branch = self.replay_minmod.pop(0) if self.replay_minmod is not None else None
            dMh = limited_gradient(M, hcv, hfp, ax, self.limiter, branch, self.record_minmod)
            S[idim] = 0.5 * dMh * _shift(hfp, 1, -1, ax)
            crop = [slice(None)] + [slice(1, -1)] * nd
            crop[ax] = slice(None)
            dMhs[idim] = dMh[tuple(crop)]
            if self.WB:
                # gradients of the equilibrium (src/muscl.py:203-204)
                dMhs[idim + nd] = limited_gradient(self.M_eq_fv, hcv, hfp, ax, self.limiter)[tuple(crop)]
        inner = (slice(None),) + (slice(1, -1),) * nd
        if self.WB:
            Mfull = M + self.M_eq_fv           # src/muscl.py:205-206
            W = Mfull[inner]
        else:
            W = M[inner]
        _p_ = nd + 1
        vels = self.vels()
        dtW = {}

        def sub(v, x):
            dtW[v] = (0.0 - x) if v not in dtW else dtW[v] - x

        for idim in range(nd):
            vel = vels[idim]
            dW = dMhs[idim]
            with np.errstate(all="ignore"):
                sub(0, W[vel] * dW[0] + W[0] * dW[vel])
                sub(_p_, W[vel] * dW[_p_] + self.gamma * W[_p_] * dW[vel])
                sub(vel, W[vel] * dW[vel] + dW[_p_] / W[0])
            if self.WB:
                # src/muscl.py:167-170; the transverse terms below then take
                # the equilibrium gradient, as the reference's reassigned dW
                dW = dMhs[idim + nd]
                sub(0, W[vel] * dW[0])
                sub(_p_, W[vel] * dW[_p_])
            for vel2 in vels[1:]:
                sub(vel2, W[vel] * dW[vel2])
        dtW[_p_] = dtW[_p_] * 0
        if self.WB:
            if self.potential:
                # src/muscl.py:208-212, on the active subcells only
                act = (slice(None),) * 0 + (slice(1, -1),) * nd
                with np.errstate(all="ignore"):
                    drho = ((Mfull[0] - self.M_eq_fv[0]) / Mfull[0])[inner[1:]]
                for vel in vels:
                    t = xp.copy(dtW[vel])
                    t[act] = t[act] + drho[act] * self.grad_phi_fv[vel - 1]
                    dtW[vel] = t
            M = Mfull - self.M_eq_fv           # src/muscl.py:214
        pred = self._embed(M, M[inner] + 0.5 * xp.stack([dtW[v] for v in range(nd + 2)], 0) * dt)
        F = {}
        for idim in range(nd):
            ax = nd - idim
            crop_m = [slice(None)] + [slice(g, -g)] * nd
            crop_s = [slice(None)] + [slice(g, -g)] * nd
            crop_m[ax] = slice(g, -1)
            crop_s[ax] = slice(1, None)
            MR = pred[tuple(crop_m)] - S[idim][tuple(crop_s)]
            crop_m[ax] = slice(1, -g)
            crop_s[ax] = slice(None, -1)
            ML = pred[tuple(crop_m)] + S[idim][tuple(crop_s)]
            if self.WB:
                # src/fv_simulator.py:150-154
                MR = MR + self.M_eq_faces[idim]
                ML = ML + self.M_eq_faces[idim]
            F[idim] = riemann(self.rs_fv, ML, MR, self.rolled_vels(idim), self.gamma,
                              self.min_c2, prims=True, iso=self.iso)
            if self.WB:
                F[idim] = F[idim] - self.F_eq_faces[idim]     # src/fv_simulator.py:163-165
        return F

    def _embed(self, M, inner):
        """M with its [1:-1]^d region replaced by ``inner``."""
        out = inner
        for idim in range(self.ndim):
            ax = self.ndim - idim
            sl = [slice(None)] + [slice(1, -1)] * self.ndim
            for k in range(idim):
                sl[self.ndim - k] = slice(None)
            lo, hi = list(sl), list(sl)
            lo[ax] = slice(0, 1)
            hi[ax] = slice(-1, None)
            out = xp.cat([M[tuple(lo)], out, M[tuple(hi)]], ax)
        return out

    def fv_update(self, F_all):
        """src/sdader_simulator.py:333-349 (with switch_to_* :288-307)."""
        nd = self.ndim
        U_cv = self.to_fv(apply_full(self.ops["sp_to_cv"], self.U_sp, nd))
        Ffaces = self.integrate_faces(F_all)
        w = self.ops["w_tp"]
        for i in range(self.T):
            W_cv = self.prims_cv(U_cv)
            dt = self.dt * w[i]
            F_HO = self.store_high_order_fluxes(Ffaces, i)
            U_new = self.fv_apply_fluxes(U_cv, F_HO, dt)
            if self.FB:
                if self.replay_affected is not None:
                    self.affected = self.replay_affected.pop(0)
                else:
                    self.detect_troubles(U_cv, U_new)
                self.record_affected.append({k: xp.copy(v) for k, v in self.affected.items()})
                F_FB = self.muscl_hancock(W_cv, dt)
                F = {}
                for idim in range(nd):
                    if self.godunov:
                        F[idim] = 1 * F_FB[idim] + (1 - 1) * F_HO[idim]
                    else:
                        theta = self.affected[idim]
                        F[idim] = theta * F_FB[idim] + (1 - theta) * F_HO[idim]
                U_new = self.fv_apply_fluxes(U_cv, F, dt)
            U_cv = U_new
        self.U_cv = self.to_sd(U_cv)
        self.U_sp = apply_full(self.ops["cv_to_sp"], self.U_cv, nd, rows=True)

    # ---- drivers (src/sdader_simulator.py:361-413) -----------------------
    def prims_cv(self, U):
        """src/sdader_simulator.py:351-356 on an FV-layout array: with WB the
        primitive perturbation prim(U + U_eq) - prim(U_eq)."""
        if self.WB:
            Ueq = self.to_fv(self.U_eq_cv)
            return (compute_primitives(U + Ueq, self.ndim, self.gamma, iso=self.iso)
                    - compute_primitives(Ueq, self.ndim, self.gamma, iso=self.iso))
        return compute_primitives(U, self.ndim, self.gamma, iso=self.iso)

    def perform_update(self):
        self.n_step += 1
        if self.WB:
            self.U_sp = self.U_sp - self.U_eq_sp
        F_all = self.ader_predictor()
        if self.update == "SD":
            self.ader_update(F_all)
        else:
            self.fv_update(F_all)
        if self.WB:
            # src/sdader_simulator.py:372-375; with the SD update U_cv is the
            # previous step's (the SD update does not recompute it)
            self.U_sp = self.U_sp + self.U_eq_sp
            self.U_cv = self.U_cv + self.U_eq_cv
        self.W_cv = compute_primitives(self.U_cv, self.ndim, self.gamma, iso=self.iso)
        self.time += self.dt

    def end_sim(self):
        self.U_cv = apply_full(self.ops["sp_to_cv"], self.U_sp, self.ndim)
        self.W_cv = compute_primitives(self.U_cv, self.ndim, self.gamma, iso=self.iso)

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
