"""The CUDA adjoint of the SD-ADER step (spd_vjp_step behind
spd_gb300.adjoint.SDADERSteps) against two references:

* torch autograd through the oracle run under torch (FP64), whose dt,
  trouble masks, theta, affected faces and minmod branches are frozen
  (detached or selected by torch.where) exactly as the CUDA adjoint freezes
  them.  Tolerance: 1e-10 relative in the 2-norm of the gradient (the two
  sum the same terms in different orders);
* central finite differences of the GPU forward with the dts and every
  decision taped and replayed (spd_tape_step), on seeded random directions
  at a generic point.  Tolerance: 1e-6 relative.
"""
import numpy as np
import pytest

from golden_cases import adjoint_case_names, case_names, load, oracle_from_golden
from gpu_helpers import product_from_golden

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


def _oracle_grad(data, kw, nsteps, w):
    """(U_sp after nsteps, dts, d<w, U_sp(nsteps)>/dU_sp(0)) from the oracle under torch autograd."""
    U0 = torch.tensor(data["init_U_sp"], dtype=torch.float64, requires_grad=True)
    o = oracle_from_golden({**data, "init_U_sp": U0}, kw)
    dts = []
    for _ in range(nsteps):
        dts.append(float(o.compute_dt()))
        o.perform_update()
    (o.U_sp * torch.tensor(w)).sum().backward()
    return o.U_sp.detach().numpy(), dts, U0.grad.numpy()


def _product_grad(s, U0, nsteps, dts, w, checkpoint_every=None):
    from spd_gb300.adjoint import run_steps
    x = torch.tensor(U0, device="cuda", requires_grad=True)
    y = run_steps(s, x, nsteps, checkpoint_every=checkpoint_every, dts=dts, refresh=False)
    (y * torch.tensor(w, device="cuda")).sum().backward()
    return y.detach().cpu().numpy(), x.grad.cpu().numpy()


def _steps_for(meta):
    return min(int(meta["steps"]), 2)


@pytest.mark.parametrize("name", adjoint_case_names())
def test_vjp_matches_torch_autograd(name):
    data, kw, meta = load(name)
    nsteps = _steps_for(meta)
    w = np.random.default_rng(7).standard_normal(data["init_U_sp"].shape)
    y_ref, dts, g_ref = _oracle_grad(data, kw, nsteps, w)
    s = product_from_golden(data, kw, meta)
    y, g = _product_grad(s, data["init_U_sp"], nsteps, dts, w)
    s.close()
    assert np.array_equal(y, y_ref)  # the forward stays bit-identical
    assert np.all(np.isfinite(g))
    rel = np.linalg.norm(g - g_ref) / np.linalg.norm(g_ref)
    assert rel < 1e-10, rel


def test_checkpoint_interval_does_not_change_the_gradient():
    """Replays from checkpoints are bit-identical, so every checkpoint
    interval gives the same gradient bit for bit."""
    data, kw, meta = load("quadrant16_p3_fvfb_hllc_gradfree")
    nsteps = 5
    w = np.random.default_rng(3).standard_normal(data["init_U_sp"].shape)
    grads = []
    dts = None
    for k in (1, 2, 5):
        s = product_from_golden(data, kw, meta)
        if dts is None:
            from spd_gb300.adjoint import AdjointRunner
            r = AdjointRunner(s, nsteps, refresh=False)
            r.forward(torch.tensor(data["init_U_sp"], device="cuda"))
            dts = r.dts
            s.close()
            s = product_from_golden(data, kw, meta)
        _, g = _product_grad(s, data["init_U_sp"], nsteps, dts, w, checkpoint_every=k)
        s.close()
        grads.append(g)
    assert np.array_equal(grads[0], grads[1]) and np.array_equal(grads[0], grads[2])


def generic_point(U0, ndim, seed, rel=1e-3):
    """U0 with seeded relative noise on density and energy and absolute
    noise (relative to density) on the momenta: a point where no
    Riemann-solver branch, limiter branch or wave-speed maximum sits
    exactly on a tie, as it does in the uniform regions of a golden
    initial state (there the frozen-branch step is not differentiable and
    central differences average the two sides of the kink)."""
    rng = np.random.default_rng(seed)
    U = np.array(U0, dtype=np.float64, copy=True)
    U[0] *= 1.0 + rel * rng.standard_normal(U[0].shape)
    U[ndim + 1] *= 1.0 + rel * rng.standard_normal(U[0].shape)
    for v in range(1, ndim + 1):
        U[v] += rel * np.abs(U[0]) * rng.standard_normal(U[0].shape)
    return U


def _fd_check(s, U0, nsteps, ndir, eps, seed):
    """Central differences of J(U) = sum(w * U_sp(nsteps)) along seeded
    entrywise-relative directions against the adjoint.  The perturbed runs
    replay the taped dts and decisions (affected faces, Riemann-solver and
    limiter branches; spd_tape_step mode 2), so both sides see the same
    frozen-decision step; returns the relative errors."""
    ctx = s._ctx
    shape = U0.shape
    rng = np.random.default_rng(seed)
    w = rng.standard_normal(shape)
    ctx.adjoint_enable(nsteps)
    ctx.tape_enable(nsteps)
    ctx.upload("U_sp", U0)
    dts = []
    for j in range(nsteps):
        dts.append(ctx.compute_dt())
        ctx.tape_step(j, dts[-1], 1)
    y = ctx.download("U_sp", shape)
    ctx.upload("U_sp", U0)
    for j in range(nsteps):
        ctx.record_step(j, dts[j])
    assert np.array_equal(ctx.download("U_sp", shape), y)
    ctx.upload("U_sp_adj", w)
    for j in range(nsteps - 1, -1, -1):
        ctx.vjp_step(j)
    g = ctx.download("U_sp_adj", shape)

    def J(x):
        ctx.upload("U_sp", x)
        for j in range(nsteps):
            ctx.tape_step(j, dts[j], 2)
        return float(np.sum(w * ctx.download("U_sp", shape)))

    assert J(U0) == float(np.sum(w * y))  # replay reproduces the recorded forward
    errs = []
    mag = np.abs(U0) + 1e-3 * np.abs(U0[0])
    for _ in range(ndir):
        v = rng.standard_normal(shape) * mag
        fd = (J(U0 + eps * v) - J(U0 - eps * v)) / (2 * eps)
        ad = float(np.sum(g * v))
        errs.append(abs(fd - ad) / max(abs(ad), 1e-300))
    return errs


@pytest.mark.parametrize("name", adjoint_case_names())
def test_vjp_matches_central_differences(name):
    data, kw, meta = load(name)
    s = product_from_golden(data, kw, meta)
    U0 = generic_point(data["init_U_sp"], len(kw["N"]), seed=5)
    errs = _fd_check(s, U0, 3, 8, 1e-7, seed=11)
    s.close()
    print(name, ["%.1e" % e for e in errs])
    assert np.median(errs) < 1e-7, errs
    assert max(errs) < 1e-6, errs


def test_batched_gradients_equal_single_instance_gradients():
    """AdjointBatch over 4 seeded Kelvin-Helmholtz instances of different
    sizes (one host thread and stream each, kernels overlapping on the GPU)
    gives each instance the gradient that instance gives alone, bit for
    bit."""
    from spd_gb300 import SDADER_Simulator
    from spd_gb300.adjoint import AdjointBatch, AdjointRunner
    from spd_gb300.initial_conditions import kelvin_helmholtz

    def make(i):
        n = (12, 16, 16, 20)[i]
        return SDADER_Simulator(p=3, N=(n, n), init_fct=kelvin_helmholtz(n, seed=500 + i), update="FV", FB=True,
                                riemann_solver_sd="hllc", riemann_solver_fv="hllc",
                                BC=(("periodic", "periodic"),) * 2, verbose=False)
    nsteps = 6
    sims = [make(i) for i in range(4)]
    U0s = [torch.tensor(s.dm.U_sp, device="cuda") for s in sims]
    ws = [torch.tensor(np.random.default_rng(40 + i).standard_normal(tuple(U.shape)), device="cuda")
          for i, U in enumerate(U0s)]
    ys, gs = AdjointBatch(sims, nsteps, checkpoint_every=2).gradients(U0s, lambda i, y: ws[i])
    for s in sims:
        s.close()
    for i in range(4):
        s = make(i)
        r = AdjointRunner(s, nsteps, checkpoint_every=2)
        y = r.forward(U0s[i])
        g = r.backward(ws[i])
        s.close()
        assert torch.equal(ys[i], y) and torch.equal(gs[i], g), i
        assert torch.isfinite(g).all()


@pytest.mark.parametrize("ndim", [1, 2, 3])
@pytest.mark.parametrize("solver", ["llf", "hllc", "lhllc"])
@pytest.mark.parametrize("update", ["SD", "FV"])
def test_taped_step_equals_plain_step(ndim, solver, update):
    """One step with every decision taped (spd_tape_step mode 1) and its
    replay (mode 2) give the plain step's state bit for bit, for every
    Riemann solver, 1D-3D, SD and FV (with limiting) updates."""
    from spd_gb300 import SDADER_Simulator
    from spd_gb300 import initial_conditions as ics
    N = {1: (16,), 2: (8, 6), 3: (4, 3, 4)}[ndim]
    s = SDADER_Simulator(p=2 if ndim == 3 else 3, N=N, init_fct=ics.sine_wave, riemann_solver_sd=solver,
                         riemann_solver_fv=solver, update=update, FB=update == "FV", verbose=False)
    ctx = s._ctx
    shape = s._shape_of("U_sp")
    U0 = generic_point(s.dm.U_sp, ndim, seed=3)
    ctx.tape_enable(1)
    ctx.upload("U_sp", U0)
    dt = ctx.compute_dt()
    ctx.set_dt(dt)
    ctx.perform_update(0.0)
    plain = ctx.download("U_sp", shape)
    out = []
    for mode in (1, 2):
        ctx.upload("U_sp", U0)
        ctx.tape_step(0, dt, mode)
        out.append(ctx.download("U_sp", shape))
    s.close()
    assert np.isfinite(plain).all()
    assert np.array_equal(out[0], plain) and np.array_equal(out[1], plain)
