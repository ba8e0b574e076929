"""Reverse-mode differentiation of SD-ADER time stepping on the GPU.

``SDADERSteps`` is a ``torch.autograd.Function`` that maps the solution-point
state ``U_sp`` (the reference's ``dm.U_sp`` layout, float64) to the state
after ``nsteps`` steps of a simulator, and whose backward pass runs the
hand-written adjoint kernels of the library (``spd_vjp_step``).

What is differentiated: each step is the map U_sp -> U_sp' with dt and every
discrete decision of the step frozen at its value in the forward pass: the
CFL dt (``SD_Simulator.compute_dt``, src/sd_simulator.py:214-227), the
trouble masks, theta and the affected faces of the a-posteriori limiter
(src/trouble_detection.py:5-87), the minmod / moncen branches of the
MUSCL-Hancock fallback (src/muscl.py:61-75) and the branches of the
LLF/HLLC Riemann solvers (src/riemann_solvers.py).  Between decisions the
step is smooth, so the gradient equals central finite differences of the
frozen-decision step.

Memory: the forward keeps a copy of U_sp every ``checkpoint_every`` steps
(default ceil(sqrt(nsteps))); the backward replays one segment at a time
from its checkpoint with the recorded dts, recording each step's
intermediates into ``checkpoint_every`` device slots, then runs the
segment's VJPs last step first.
"""
from __future__ import annotations

import math

import torch

__all__ = ["SDADERSteps", "AdjointRunner", "AdjointBatch", "run_steps"]


def _sync(t: torch.Tensor):
    """Wait for the work queued on ``t``'s device by this thread's current
    torch stream (the library's own stream is synchronised by each call)."""
    if t.is_cuda:
        torch.cuda.current_stream(t.device).synchronize()


class AdjointRunner:
    """Forward and backward passes of ``nsteps`` steps of one simulator.

    The simulator's device state is overwritten by both passes; after
    ``forward`` it holds the final state and ``sim.time`` / ``sim.n_step``
    are advanced; the backward pass leaves it at an intermediate step.
    ``dts`` (optional) fixes the step sizes instead of the CFL reduction.
    With ``refresh`` the subcell averages and primitives that the first CFL
    reduction reads are recomputed from ``U0`` (as ``end_sim`` does);
    without it they are the simulator's current ones, as when the
    reference's ``dm.U_sp`` is assigned."""

    def __init__(self, sim, nsteps: int, checkpoint_every: int | None = None, dts=None, refresh: bool = True):
        if nsteps < 1:
            raise ValueError("nsteps must be >= 1")
        self.sim = sim
        self.ctx = sim._ctx
        self.nsteps = int(nsteps)
        self.k = int(checkpoint_every or math.ceil(math.sqrt(self.nsteps)))
        self.k = max(1, min(self.k, self.nsteps))
        self.refresh = bool(refresh)
        self.fixed_dts = None if dts is None else [float(x) for x in dts]
        if self.fixed_dts is not None and len(self.fixed_dts) != self.nsteps:
            raise ValueError("dts must hold one value per step")
        self.shape = sim._shape_of("U_sp")
        self.count = math.prod(self.shape)
        self.dts: list[float] = []
        self.checkpoints: list[torch.Tensor] = []
        self.device = torch.device("cuda") if torch.cuda.is_available() else torch.device("cpu")

    # -- state transfer (host or device tensors; the library copies with
    #    cudaMemcpyDefault) ------------------------------------------------
    def _put(self, field: str, x: torch.Tensor):
        x = x.detach().to(torch.float64).contiguous()
        if tuple(x.shape) != tuple(self.shape):
            raise ValueError(f"{field}: expected shape {self.shape}, got {tuple(x.shape)}")
        _sync(x)
        self.ctx.upload_ptr(field, x.data_ptr(), self.count)

    def _get(self, field: str, device=None) -> torch.Tensor:
        out = torch.empty(self.shape, dtype=torch.float64, device=device or self.device)
        _sync(out)
        self.ctx.download_ptr(field, out.data_ptr(), self.count)
        return out

    def forward(self, U0: torch.Tensor) -> torch.Tensor:
        self._put("U_sp", U0)
        if self.refresh:
            # U_cv and W_cv (the CFL reduction's input) from the new state
            self.ctx.end_sim()
        self.dts = []
        self.checkpoints = []
        time = self.sim.time
        for j in range(self.nsteps):
            if j % self.k == 0:
                self.checkpoints.append(self._get("U_sp"))
            if self.fixed_dts is None:
                dt = self.ctx.compute_dt()
            else:
                dt = self.fixed_dts[j]
                self.ctx.set_dt(dt)
            time = self.ctx.perform_update(time)
            self.dts.append(dt)
        self.sim.time = time
        self.sim.n_step += self.nsteps
        return self._get("U_sp", device=U0.device)

    def backward(self, grad_out: torch.Tensor) -> torch.Tensor:
        if len(self.dts) != self.nsteps:
            raise RuntimeError("backward before forward")
        self.ctx.adjoint_enable(self.k)
        self._put("U_sp_adj", grad_out)
        nseg = len(self.checkpoints)
        for s in range(nseg - 1, -1, -1):
            start = s * self.k
            stop = min(start + self.k, self.nsteps)
            self._put("U_sp", self.checkpoints[s])
            for j in range(start, stop):
                self.ctx.record_step(j - start, self.dts[j])
            for j in range(stop - 1, start - 1, -1):
                self.ctx.vjp_step(j - start)
        return self._get("U_sp_adj", device=grad_out.device)


class SDADERSteps(torch.autograd.Function):
    """U_sp(0) -> U_sp(nsteps) with a GPU adjoint; see the module docstring."""

    @staticmethod
    def forward(ctx, U0: torch.Tensor, runner: AdjointRunner):  # noqa: D401
        ctx.runner = runner
        return runner.forward(U0)

    @staticmethod
    def backward(ctx, grad_out):
        return ctx.runner.backward(grad_out), None


def run_steps(sim, U0: torch.Tensor, nsteps: int, checkpoint_every: int | None = None, dts=None,
              refresh: bool = True) -> torch.Tensor:
    """Differentiable ``nsteps`` steps of ``sim`` starting from ``U0``."""
    return SDADERSteps.apply(U0, AdjointRunner(sim, nsteps, checkpoint_every, dts, refresh))


class AdjointBatch:
    """Gradients of many independent simulators at once.

    Each instance keeps its own context, CUDA stream and ``AdjointRunner``;
    one host thread per instance issues its forward and backward passes, so
    the instances' kernels overlap on the GPU while every call of the
    library still waits only for its own stream.  Every instance's result
    is the one its ``AdjointRunner`` gives alone (the same launches on the
    same data, bit for bit)."""

    def __init__(self, sims, nsteps: int, checkpoint_every: int | None = None, dts=None, refresh: bool = True,
                 max_workers: int | None = None):
        if not sims:
            raise ValueError("AdjointBatch needs at least one simulator")
        if len({id(s._ctx) for s in sims}) != len(sims):
            raise ValueError("AdjointBatch: every instance needs its own simulator (context)")
        per = [None] * len(sims) if dts is None else list(dts)
        if len(per) != len(sims):
            raise ValueError("dts: one list per instance")
        self.runners = [AdjointRunner(s, nsteps, checkpoint_every, d, refresh) for s, d in zip(sims, per)]
        self.max_workers = int(max_workers or len(sims))

    def _map(self, fn, items):
        import concurrent.futures
        with concurrent.futures.ThreadPoolExecutor(max_workers=self.max_workers) as ex:
            return list(ex.map(fn, range(len(self.runners)), items))

    def forward(self, U0s):
        """Final states of every instance (one tensor per instance)."""
        if len(U0s) != len(self.runners):
            raise ValueError("one initial state per instance")
        return self._map(lambda i, U0: self.runners[i].forward(U0), U0s)

    def backward(self, grads_out):
        """Gradients with respect to every instance's initial state."""
        if len(grads_out) != len(self.runners):
            raise ValueError("one output gradient per instance")
        return self._map(lambda i, g: self.runners[i].backward(g), grads_out)

    def gradients(self, U0s, loss_grad):
        """forward, ``loss_grad(i, y_i) -> dJ/dy_i`` and backward of every
        instance in its own thread (no instance waits for another's
        forward); returns (final states, gradients)."""
        if len(U0s) != len(self.runners):
            raise ValueError("one initial state per instance")

        def one(i, U0):
            y = self.runners[i].forward(U0)
            return y, self.runners[i].backward(loss_grad(i, y))
        out = self._map(one, U0s)
        return [o[0] for o in out], [o[1] for o in out]
