"""Host logic of the checkpointed adjoint (spd_gb300.adjoint) on a CPU
stand-in for the library context: every step is an affine map
x -> M_j x + c_j chosen by the step's dt, record/VJP slots behave like the
library's, and the gradient that the segment replays assemble must equal
the product of the transposed step matrices for every checkpoint interval."""
import ctypes

import numpy as np
import pytest

torch = pytest.importorskip("torch")


def _view(ptr, count):
    return np.ctypeslib.as_array((ctypes.c_double * count).from_address(ptr))


class FakeCtx:
    """The subset of spd_gb300._lib.Context used by AdjointRunner."""

    def __init__(self, mats, shifts, dts):
        self.mats, self.shifts, self.dts = mats, shifts, dts
        self.x = None
        self.adj = None
        self.dt = None
        self.slots = {}
        self.depth = 0
        self.calls = []
        self.nstep = 0

    def upload_ptr(self, field, ptr, count):
        data = _view(ptr, count).copy()
        if field == "U_sp":
            self.x = data
        elif field == "U_sp_adj":
            self.adj = data
        else:
            raise KeyError(field)

    def download_ptr(self, field, ptr, count):
        _view(ptr, count)[:] = self.x if field == "U_sp" else self.adj

    def end_sim(self):
        pass

    def compute_dt(self):
        self.dt = self.dts[self.nstep % len(self.dts)]
        return self.dt

    def set_dt(self, dt):
        self.dt = dt

    def _apply(self, dt):
        j = self.dts.index(dt)
        self.x = self.mats[j] @ self.x + self.shifts[j]
        return j

    def perform_update(self, time):
        self._apply(self.dt)
        self.nstep += 1
        return time + self.dt

    def adjoint_enable(self, depth):
        self.depth = max(self.depth, depth)

    def record_step(self, slot, dt):
        assert 0 <= slot < self.depth
        self.slots[slot] = self._apply(dt)
        self.calls.append(("record", slot))

    def vjp_step(self, slot):
        self.adj = self.mats[self.slots[slot]].T @ self.adj
        self.calls.append(("vjp", slot))


class FakeSim:
    def __init__(self, ctx, shape):
        self._ctx = ctx
        self.shape = shape
        self.time = 0.0
        self.n_step = 0

    def _shape_of(self, name):
        assert name == "U_sp"
        return self.shape


@pytest.mark.parametrize("k", [None, 1, 2, 3, 7, 11])
def test_checkpointed_gradient_equals_the_transposed_product(k):
    from spd_gb300.adjoint import run_steps
    rng = np.random.default_rng(4)
    shape = (3, 2, 2)
    n = int(np.prod(shape))
    nsteps = 11
    mats = [np.eye(n) + 0.1 * rng.standard_normal((n, n)) for _ in range(nsteps)]
    shifts = [rng.standard_normal(n) for _ in range(nsteps)]
    dts = [1e-3 * (j + 1) for j in range(nsteps)]
    sim = FakeSim(FakeCtx(mats, shifts, dts), shape)
    x0 = torch.tensor(rng.standard_normal(shape), dtype=torch.float64, requires_grad=True)
    y = run_steps(sim, x0, nsteps, checkpoint_every=k)
    ref = x0.detach().numpy().reshape(-1)
    for j in range(nsteps):
        ref = mats[j] @ ref + shifts[j]
    assert np.allclose(y.detach().numpy().reshape(-1), ref, rtol=0, atol=1e-12)
    w = torch.tensor(rng.standard_normal(shape))
    (y * w).sum().backward()
    g = w.numpy().reshape(-1)
    for j in reversed(range(nsteps)):
        g = mats[j].T @ g
    assert np.allclose(x0.grad.numpy().reshape(-1), g, rtol=1e-12, atol=1e-12)
    assert sim.time == pytest.approx(sum(dts)) and sim.n_step == nsteps
    # every VJP is applied to the slot recorded for its step, last step first
    vjps = [slot for kind, slot in sim._ctx.calls if kind == "vjp"]
    assert len(vjps) == nsteps


def test_fixed_dts_are_replayed():
    from spd_gb300.adjoint import AdjointRunner
    rng = np.random.default_rng(5)
    shape = (2, 3)
    n = 6
    mats = [np.eye(n) + 0.05 * rng.standard_normal((n, n)) for _ in range(4)]
    shifts = [np.zeros(n)] * 4
    dts = [0.5, 0.25, 0.125, 0.0625]
    sim = FakeSim(FakeCtx(mats, shifts, dts), shape)
    r = AdjointRunner(sim, 4, checkpoint_every=2, dts=dts[::-1])
    r.forward(torch.zeros(shape, dtype=torch.float64))
    assert r.dts == dts[::-1]
    with pytest.raises(ValueError):
        AdjointRunner(sim, 3, dts=[0.1])


def test_adjoint_batch_equals_each_instance_alone():
    """AdjointBatch (one host thread per instance) gives every instance the
    gradient its AdjointRunner gives alone."""
    from spd_gb300.adjoint import AdjointBatch, AdjointRunner
    rng = np.random.default_rng(6)
    shape = (2, 2, 2)
    n = 8
    nsteps = 5
    problems = []
    for b in range(4):
        mats = [np.eye(n) + 0.1 * rng.standard_normal((n, n)) for _ in range(nsteps)]
        shifts = [rng.standard_normal(n) for _ in range(nsteps)]
        dts = [1e-3 * (j + 1 + 10 * b) for j in range(nsteps)]
        problems.append((mats, shifts, dts))
    U0s = [torch.tensor(rng.standard_normal(shape)) for _ in problems]
    ws = [torch.tensor(rng.standard_normal(shape)) for _ in problems]
    batch = AdjointBatch([FakeSim(FakeCtx(*pr), shape) for pr in problems], nsteps, checkpoint_every=2)
    ys, gs = batch.gradients(U0s, lambda i, y: ws[i])
    for i, pr in enumerate(problems):
        r = AdjointRunner(FakeSim(FakeCtx(*pr), shape), nsteps, checkpoint_every=2)
        y = r.forward(U0s[i])
        g = r.backward(ws[i])
        assert torch.equal(ys[i], y) and torch.equal(gs[i], g)
    with pytest.raises(ValueError):
        batch.forward(U0s[:2])
    sim = FakeSim(FakeCtx(*problems[0]), shape)
    with pytest.raises(ValueError):
        AdjointBatch([sim, sim], nsteps)
