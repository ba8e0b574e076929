"""Algorithmic FP64 operation count of the SD-ADER step -- MEASUREMENT
INFRASTRUCTURE ONLY (used by tests/; the product never imports it).

Runs the oracle restatement (``oracle/sdader_oracle.py``, which follows the
reference's operation order) on torch FP64 tensors under a
``TorchFunctionMode`` that counts, per element of every FP64 result, the
additions/subtractions, multiplications, divisions and square roots (a
square by ``x ** 2`` counts as one multiplication; negation, |x|, maxima,
minima, selections and comparisons are not floating-point operations and
are not counted).  Each count is attributed to a phase: the innermost
oracle method being executed, with a per-step call index (the k-th
``solve_faces`` of a step is the k-th Picard iteration), and the outermost
oracle function called from it (``apply_axis`` = a 1D operator
contraction, ``compute_primitives``/``compute_fluxes`` = the Euler maps,
``riemann`` = an interface solve with everything it calls).

    python -m oracle.flop_count [ndim p N]

prints the count per cell and step of every phase.
"""
from __future__ import annotations

import collections
import functools
import sys

import numpy as np

from . import sdader_oracle as so

try:
    import torch
    from torch.overrides import TorchFunctionMode
except Exception:  # pragma: no cover
    torch = None
    TorchFunctionMode = object

_KIND = {}
for _n in ("add", "__add__", "__radd__", "__iadd__", "sub", "__sub__", "__rsub__", "__isub__", "subtract"):
    _KIND[_n] = "add"
for _n in ("mul", "__mul__", "__rmul__", "__imul__", "multiply"):
    _KIND[_n] = "mul"
for _n in ("div", "true_divide", "__truediv__", "__rtruediv__", "__itruediv__", "divide"):
    _KIND[_n] = "div"
_KIND["sqrt"] = "sqrt"

FUNCTIONS = ("apply_axis", "apply_full", "compute_primitives", "compute_conservatives", "compute_fluxes",
             "compute_cs", "riemann", "limited_gradient", "minmod", "minmod_branch", "moncen")
METHODS = ("compute_dt", "solve_faces", "ader_dudt", "ader_predictor", "ader_update", "fv_update",
           "fv_apply_fluxes", "detect_troubles", "muscl_hancock", "integrate_faces", "store_high_order_fluxes",
           "fv_boundaries", "end_sim", "perform_update")


class Counter(TorchFunctionMode):
    def __init__(self):
        super().__init__()
        self.counts = collections.Counter()
        self.methods = []      # stack of (method, call index)
        self.functions = []    # stack of function names
        self.calls = collections.Counter()

    def phase(self):
        meth = "%s[%d]" % self.methods[-1] if self.methods else "-"
        fn = self.functions[0] if self.functions else "-"
        return meth + "/" + fn

    def __torch_function__(self, func, types, args=(), kwargs=None):
        out = func(*args, **(kwargs or {}))
        name = getattr(func, "__name__", "")
        kind = _KIND.get(name)
        if name in ("pow", "__pow__") and len(args) > 1 and args[1] == 2:
            kind = "mul"
        if kind and torch.is_tensor(out) and out.dtype == torch.float64:
            self.counts[(self.phase(), kind)] += out.numel()
        return out


def _wrap_function(counter, fn):
    @functools.wraps(fn)
    def w(*a, **k):
        counter.functions.append(fn.__name__)
        try:
            return fn(*a, **k)
        finally:
            counter.functions.pop()
    return w


def _wrap_method(counter, fn):
    @functools.wraps(fn)
    def w(self, *a, **k):
        if fn.__name__ == "perform_update":
            counter.calls.clear()
        idx = counter.calls[fn.__name__]
        counter.calls[fn.__name__] += 1
        counter.methods.append((fn.__name__, idx))
        saved, counter.functions = counter.functions, []
        try:
            return fn(self, *a, **k)
        finally:
            counter.functions = saved
            counter.methods.pop()
    return w


def count_step(oracle_kwargs: dict) -> dict:
    """FP64 operations of one compute_dt + perform_update of an oracle built
    from ``oracle_kwargs`` (state arrays as NumPy), per phase and kind:
    {(phase, kind): count}."""
    if torch is None:
        raise RuntimeError("torch is needed for the operation count")
    counter = Counter()
    saved_f = {n: getattr(so, n) for n in FUNCTIONS}
    saved_m = {n: getattr(so.OracleSDADER, n) for n in METHODS}
    try:
        for n in FUNCTIONS:
            setattr(so, n, _wrap_function(counter, saved_f[n]))
        for n in METHODS:
            setattr(so.OracleSDADER, n, _wrap_method(counter, saved_m[n]))
        kw = dict(oracle_kwargs)
        kw["state"] = {k: torch.as_tensor(np.asarray(v, dtype=np.float64)) for k, v in kw["state"].items()}
        o = so.OracleSDADER(**kw)
        with counter:
            o.compute_dt()
            o.perform_update()
    finally:
        for n, f in saved_f.items():
            setattr(so, n, f)
        for n, f in saved_m.items():
            setattr(so.OracleSDADER, n, f)
    return dict(counter.counts)


def oracle_kwargs_for(ndim, p, N, update="FV", FB=True, rs="hllc", seed=0):
    """A smooth periodic state (every subcell troubled-free is not needed:
    the predictor's count does not depend on the data) for the count."""
    sys_path_root = __file__.rsplit("/oracle/", 1)[0]
    if sys_path_root not in sys.path:
        sys.path.insert(0, sys_path_root)
    from spd_gb300.simulator import SDADER_Simulator, initial_state
    from spd_gb300 import initial_conditions as ics
    ops = SDADER_Simulator.build_operators(p, p)
    Ns = [N] * ndim
    lims = [(0.0, 1.0)] * ndim
    _, W_cv, _, U_sp, U_cv = initial_state(ndim, Ns, p, lims, ics.sine_wave, ops, 1.4)
    state = {"U_sp": U_sp, "U_cv": U_cv, "W_cv": W_cv.copy()}
    for i, d in enumerate("xyz"[:ndim]):
        T = p + 1
        state[f"BC_fp_{d}"] = np.zeros((2, ndim + 2, T) + tuple([N] * (ndim - 1)) + (p + 1,) * (ndim - 1))
        ext = [N * (p + 1) + 4] * ndim
        ext[i] = 2
        state[f"BC_fv_{d}"] = np.zeros((2, ndim + 2) + tuple(ext[::-1]))
    return dict(ndim=ndim, N=Ns, p=p, m=p, lims=lims, BC=[("periodic", "periodic")] * ndim, gamma=1.4,
                cfl_coeff=0.8, min_c2=1e-10, riemann_solver_sd=rs, riemann_solver_fv=rs, slope_limiter="minmod",
                update=update, FB=FB, tolerance=1e-5, SED=True, NAD="", PAD=True, blending=True, min_rho=1e-10,
                max_rho=1e10, min_P=1e-10, godunov=False, ops=ops, state=state)


def per_cell(counts: dict, cells: int) -> dict:
    out = collections.defaultdict(dict)
    for (phase, kind), c in counts.items():
        out[phase][kind] = c / cells
    return dict(out)


if __name__ == "__main__":
    nd, p, N = (int(x) for x in sys.argv[1:4]) if len(sys.argv) > 3 else (2, 3, 4)
    res = per_cell(count_step(oracle_kwargs_for(nd, p, N)), N ** nd)
    for phase in sorted(res):
        tot = sum(res[phase].values())
        print(f"{phase:45s} {tot:12.1f}  " + " ".join(f"{k}={v:g}" for k, v in sorted(res[phase].items())))
