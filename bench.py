"""Throughput of the GB300 SD-ADER step: FP64 DOF-updates/s.

Default workload: the four-quadrant 2D Riemann problem on [0,1]^2 with
transmissive boundaries, 512x512 cells, p=3 (16 solution points per cell),
HLLC, NAD/SED/PAD trouble detection with MUSCL-Hancock fallback on
(p+1)^2 subcells.  One step = compute_dt + perform_update (the body of
SDADER_Simulator.perform_iterations).  DOF = cells * (p+1)^2.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Prints one JSON line.  ``--impl reference`` times the CPU restatement of the
reference's NumPy path on the host cores (one independent instance per
core) on a bounded sample of the same configuration.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "FP64 DOF-updates/s on 1 GB300 (p=3)"
UNIT = "DOF-updates/s"

WORKLOADS = {
    # name: (description, constructor kwargs factory)
    "quadrant512": "four-quadrant Riemann problem, 512x512 cells, p=3, FV update with NAD/SED/PAD limiting and "
                   "MUSCL-Hancock fallback, HLLC, transmissive boundaries",
    "vortex32": "isentropic vortex, 32x32 cells, p=3, FV update with limiting, LLF, periodic",
    "sedov128": "3D Sedov blast, 128^3 cells, p=2, FV update with limiting, HLLC, reflective",
    "vortex512_sd": "isentropic vortex on [0,10]^2, 512x512 cells, p=3, SD update (no limiter), LLF, periodic",
    "quadrant512_lhllc_moncen": "four-quadrant Riemann problem, 512x512 cells, p=3, FV update with limiting, "
                                "low-Mach HLLC, moncen slopes, transmissive boundaries",
    "kh_ensemble_small": "batched: 256 periodic Kelvin-Helmholtz shear layers, p=3, sides drawn from "
                         "{16,24,32,48,64} (seed 2026), HLLC + limiting, per-instance dt",
    "kh_ensemble": "batched: 64 periodic Kelvin-Helmholtz shear layers, p=3, sides drawn from "
                   "{64,128,192,256,384,512} (seed 2026), HLLC + limiting, per-instance dt",
    "kh_adjoint": "gradient of J = ||rho(T) - rho_target||^2 with respect to the initial density, periodic "
                  "Kelvin-Helmholtz shear layer, 256x256 cells, p=3, 200 steps, HLLC + limiting (masks, "
                  "branches and dt frozen from the forward), sqrt(N) checkpoints; rho_target from a forward run "
                  "of a seeded 1e-2 Gaussian density perturbation",
}


def workload_kwargs(name, n_override=None):
    from spd_gb300 import initial_conditions as ics
    if name == "quadrant512":
        n = n_override or 512
        return dict(p=3, N=(n, n), init_fct=ics.four_quadrant, update="FV", FB=True, riemann_solver_sd="hllc",
                    riemann_solver_fv="hllc", BC=(("gradfree", "gradfree"),) * 2, cfl_coeff=0.8)
    if name == "vortex32":
        n = n_override or 32
        return dict(p=3, N=(n, n), xlim=(0, 10), ylim=(0, 10), init_fct=ics.isentropic_vortex(), update="FV",
                    FB=True, riemann_solver_sd="llf", riemann_solver_fv="llf", BC=(("periodic", "periodic"),) * 2)
    if name == "vortex512_sd":
        n = n_override or 512
        return dict(p=3, N=(n, n), xlim=(0, 10), ylim=(0, 10), init_fct=ics.isentropic_vortex(), update="SD",
                    riemann_solver_sd="llf", BC=(("periodic", "periodic"),) * 2)
    if name == "quadrant512_lhllc_moncen":
        n = n_override or 512
        return dict(p=3, N=(n, n), init_fct=ics.four_quadrant, update="FV", FB=True, riemann_solver_sd="lhllc",
                    riemann_solver_fv="lhllc", slope_limiter="moncen", BC=(("gradfree", "gradfree"),) * 2,
                    cfl_coeff=0.8)
    if name == "sedov128":
        n = n_override or 128
        return dict(p=2, N=(n, n, n), init_fct=ics.sedov(n), update="FV", FB=True, riemann_solver_sd="hllc",
                    riemann_solver_fv="hllc", BC=(("reflective", "reflective"),) * 3)
    raise KeyError(name)


def dof_of(kw):
    cells = 1
    for n in kw["N"]:
        cells *= n
    return cells * (kw["p"] + 1) ** len(kw["N"]), cells


# ---------------------------------------------------------------------------
# clocks during the timed region
# ---------------------------------------------------------------------------
class ClockSampler:
    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index=0):
        self.path = tempfile.mktemp(suffix=".csv")
        self.proc = None
        self.gpu = gpu_index

    def __enter__(self):
        try:
            self.fh = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.QUERY}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=self.fh, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
            self.fh.close()

    def summary(self):
        if self.proc is None or not os.path.exists(self.path):
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unavailable"]}
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax = float(f[2])
            except ValueError:
                continue
            for k, name in enumerate(names):
                if f[5 + k].lower() == "active":
                    reasons.add(name)
        os.unlink(self.path)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": smax, "reasons": sorted(reasons),
                "samples": len(sm)}


# ---------------------------------------------------------------------------
# roofline bookkeeping
# ---------------------------------------------------------------------------
def measured_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        d = json.load(open(path))
        return d.get("hbm_gbs", 6800.0), "measured"
    return 6800.0, "fallback"


def interior_flops_per_cell_step(D, p, m, update):
    """Algorithmic FP64 operations of the work of all k_interior launches of
    one step, per cell (one operation per add, subtract, multiply, divide;
    a square root would count one): the reference's own arithmetic for that
    work, counted once -- the sp -> fp interpolation of the interior flux
    points and the edge traces (src/transforms.py:3-25), U -> W and the Euler
    flux at interior flux points (src/hydro.py:48-86,127-170), the flux
    derivative and its division by h (src/sd_simulator.py:196-206), the
    Picard update (src/sdader_simulator.py:194-200) and, with update="SD",
    the final weighted update (:202-208).  The first Picard iteration's T
    time nodes are equal and count once (the reference evaluates them T
    times).  The per-point terms equal the instrumented oracle's counts
    (oracle/flop_count.py, checked by tests/test_flop_count.py)."""
    n, nf, V, T = p + 1, p + 2, D + 2, m + 1
    NS, NJ = n ** D, n ** (D - 1)
    interp = 2 * n - 1                      # one flux-point value of one variable
    prim = 3 * D + 3                        # U -> W at one point
    flux = 4 * D + 6                        # Euler flux at one point
    faces = D * NJ * (nf - 2) * (V * interp + prim + flux)    # interior flux points of one time node
    dudt = V * NS * (D * 2 * nf + (D - 1))                       # sum_d dfp_to_sp(F)/h of one time node
    picard = V * NS * T * (2 * T + 1)                            # invader contraction, *dt, U_sp -
    traces = D * NJ * 2 * V * interp                             # edge traces of one time node
    sd_update = V * NS * (2 * T + 1)                             # w_tp contraction, *dt, U_sp -
    total = 0
    for it in range(m + 1):
        teff = 1 if it == 0 else T
        total += faces * teff
        if it < m:
            total += dudt * teff + picard + traces * T
        elif update == "SD":
            total += dudt * teff + sd_update
    return total


def compulsory_bytes_per_cell_step(D, p):
    """Compulsory HBM traffic of a step per cell: U_sp read and written once
    (2 * V * (p+1)^D doubles)."""
    return 2 * (D + 2) * (p + 1) ** D * 8


# DRAM traffic (read + write bytes) and executed FP64 instructions (DADD +
# DMUL + DFMA, thread level) of k_interior per cell and step, summed over
# the (m+1) launches of a step; 2D, p = 3, FV update.  Source: one ncu
# capture, --clock-control none -k regex:k_interior over the four launches of
# one step, metrics dram__bytes_read.sum, dram__bytes_write.sum,
# smsp__sass_thread_inst_executed_op_{dadd,dmul,dfma}_pred_on.sum, of
# `python bench.py --lean --cells 256 --steps 1 --warmup 1 [--build fma]`,
# divided by the 65,536 cells (both scale with the cell count, and h = 1/256
# is a power of two as at 512^2, so the derivative takes the same
# prescaled form; the full 512^2 workload is not captured with more than
# one pass).  Keyed by (D, p, update, build).
NCU_K_INTERIOR = {
    (2, 3, "FV", "ieee"): {"cells_captured": 256 * 256, "dram_bytes": 12085.9 + 14239.4, "fp64_inst": 42043.0},
    (2, 3, "FV", "fma"): {"cells_captured": 256 * 256, "dram_bytes": 12122.4 + 14251.4, "fp64_inst": 28651.0},
}


def fp64_peak_tflops():
    """cuBLAS FP64 GEMM throughput (burst), the FP64 denominator."""
    import torch
    n = 8192
    a = torch.randn(n, n, dtype=torch.float64, device="cuda")
    b = torch.randn(n, n, dtype=torch.float64, device="cuda")
    torch.matmul(a, b)
    torch.cuda.synchronize()
    best = 1e30
    for _ in range(3):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        torch.matmul(a, b)
        e1.record()
        torch.cuda.synchronize()
        best = min(best, e0.elapsed_time(e1) / 1e3)
    del a, b
    return 2 * n ** 3 / best / 1e12


# ---------------------------------------------------------------------------
# CPU baseline: the oracle restatement of the reference's NumPy path
# ---------------------------------------------------------------------------
def _cpu_worker(args):
    workload, n_side, steps, warmup = args[:4]
    want_state = len(args) > 4 and args[4]
    os.environ.setdefault("OMP_NUM_THREADS", "1")
    sys.path.insert(0, ROOT)
    import warnings
    warnings.simplefilter("ignore")
    import numpy as np
    from oracle.sdader_oracle import OracleSDADER
    from spd_gb300.simulator import SDADER_Simulator, initial_state, subcell_faces  # noqa: F401
    kw = workload_kwargs(workload, n_side)
    ndim = len(kw["N"])
    p = kw["p"]
    ops = SDADER_Simulator.build_operators(p, p)
    lims = [kw.get(f"{d}lim", (0, 1)) for d in "xyz"[:ndim]]
    _, W_cv, _, U_sp, U_cv = initial_state(ndim, list(kw["N"]), p, lims, kw["init_fct"], ops, 1.4)
    state = {"U_sp": U_sp, "U_cv": U_cv, "W_cv": W_cv.copy()}
    for d in "xyz"[:ndim]:
        state[f"BC_fp_{d}"] = np.zeros(1)
        ext = [kw["N"][i] * (p + 1) + 4 for i in range(ndim)]
        ext["xyz".index(d)] = 2
        state[f"BC_fv_{d}"] = np.zeros((2, ndim + 2) + tuple(ext[::-1]))
    o = OracleSDADER(ndim=ndim, N=list(kw["N"]), p=p, m=p, lims=lims, BC=kw["BC"], gamma=1.4,
                     cfl_coeff=kw.get("cfl_coeff", 0.8), min_c2=1e-10, riemann_solver_sd=kw["riemann_solver_sd"],
                     riemann_solver_fv=kw.get("riemann_solver_fv", "llf"),
                     slope_limiter=kw.get("slope_limiter", "minmod"), update=kw["update"],
                     FB=kw.get("FB", False), tolerance=1e-5, SED=True, NAD="", PAD=True, blending=True, min_rho=1e-10,
                     max_rho=1e10, min_P=1e-10, godunov=False, ops=ops, state=state)
    for _ in range(warmup):
        o.compute_dt()
        o.perform_update()
    t0 = time.perf_counter()
    for _ in range(steps):
        o.compute_dt()
        o.perform_update()
    el = time.perf_counter() - t0
    dof, _ = dof_of(kw)
    if want_state:
        return dof * steps, el, np.asarray(o.U_sp)
    return dof * steps, el


def cpu_baseline(workload, n_side, steps, warmup, procs, want_state=False):
    import multiprocessing as mp
    ctx = mp.get_context("spawn")
    with ctx.Pool(procs) as pool:
        res = pool.map(_cpu_worker, [(workload, n_side, steps, warmup, want_state)] * procs)
    total_units = sum(r[0] for r in res)
    tmax = max(r[1] for r in res)
    if want_state:
        return total_units / tmax, tmax, res[0][2]
    return total_units / tmax, tmax


def sample_parity(workload, n_side, U_oracle):
    """The same sample (n_side cells per direction, one step from the
    initial state) on the GPU against the oracle's U_sp."""
    import numpy as np
    from spd_gb300 import SDADER_Simulator
    s = SDADER_Simulator(verbose=False, **workload_kwargs(workload, n_side))
    s.compute_dt()
    s.perform_update()
    U = s.dm.U_sp
    s.close()
    dev = np.abs(U - U_oracle)
    rel = dev / np.maximum(np.abs(U_oracle), 1e-300)
    ndim = (U.ndim - 1) // 2
    return {"sample": "x".join([str(n_side)] * ndim) + " cells, 1 step from the initial state",
            "max_abs_dev": float(np.nanmax(dev)), "max_rel_dev": float(np.nanmax(rel)),
            "bitwise_equal": bool(np.array_equal(U, U_oracle, equal_nan=True))}


def vortex_t1_error():
    """The vortex configuration (32x32 cells on [0,10]^2, p=3, LLF, FV with
    limiting) run to t=1: L1 error of the subcell-averaged density against
    the exact translated vortex."""
    import numpy as np
    from spd_gb300 import SDADER_Simulator
    from spd_gb300.initial_conditions import isentropic_vortex
    from spd_gb300.polynomials import quadrature_mean
    s = SDADER_Simulator(verbose=False, **workload_kwargs("vortex32"))
    s.perform_time_evolution(1.0)
    exact = s.crop(quadrature_mean(s.mesh_cv, isentropic_vortex(center=(6.0, 6.0)), 2, 0, light=False)[None])[0]
    err = float(np.mean(np.abs(s.dm.W_cv[0] - exact)))
    out = {"t_end": 1.0, "steps": s.n_step, "l1_density_error_vs_exact": err}
    s.close()
    return out


def other_configs(args, steps=5):
    """The other single-GPU configurations timed like the headline (compute_dt
    + perform_update per step, launch by launch, CUDA events on the
    library's stream after 3 warm-up steps) and through the graph driver
    (perform_iterations: one captured step replayed): the vortex 32^2 (p=3,
    FV with limiting, LLF) and the 3D Sedov blast 128^3 (p=2, FV with
    limiting, HLLC), each with its own clock record."""
    import torch
    from spd_gb300 import SDADER_Simulator
    out = {}
    for name in ("vortex32", "sedov128"):
        kw = workload_kwargs(name)
        dof, cells = dof_of(kw)
        s = SDADER_Simulator(verbose=False, fma=args.build == "fma", **kw)
        stream = torch.cuda.current_stream()
        s._ctx.set_stream(stream.cuda_stream)
        for _ in range(3):
            s.compute_dt()
            s.perform_update()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        with ClockSampler(0) as clk:
            e0.record(stream)
            for _ in range(steps):
                s.compute_dt()
                s.perform_update()
            e1.record(stream)
            torch.cuda.synchronize()
        ms = e0.elapsed_time(e1)
        s.time, _, _ = s._ctx.step(1, 0.0, 0, s.time)  # graph capture (untimed)
        torch.cuda.synchronize()
        g0, g1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        g0.record(stream)
        s.time, _, _ = s._ctx.step(steps, 0.0, 0, s.time)
        g1.record(stream)
        torch.cuda.synchronize()
        gms = g0.elapsed_time(g1)
        s.close()
        out[name] = {"workload": WORKLOADS[name], "cells": cells, "dof": dof, "steps": steps, "warmup": 3,
                     "ms_per_step": ms / steps, "value": dof * steps / (ms / 1e3), "unit": UNIT,
                     "graph_driver": {"ms_per_step": gms / steps, "value": dof * steps / (gms / 1e3)},
                     "clocks": clk.summary(),
                     "l2": ("inputs smaller than L2 (launch-bound case)" if name == "vortex32"
                            else "inputs larger than L2")}
    return out


FULL_RUNS = {
    # workload: (what the configuration runs to, driver)
    "quadrant512": ("t_end", 0.8),
    "sedov128": ("steps", 200),
    "vortex32": ("t_end", 1.0),
    "vortex512_sd": ("steps", 200),
    "quadrant512_lhllc_moncen": ("t_end", 0.8),
}


def full_run_arm(args):
    """The workload's whole run as its configuration specifies it (the
    four-quadrant problem to t=0.8, the Sedov blast for 200 steps, ...)
    through the reference's drivers (perform_time_evolution /
    perform_iterations: one captured step replayed per step), timed with
    CUDA events: steps, time to solution, DOF-updates/s over the run, and
    the state's health at the end (finite, trouble count)."""
    import numpy as np
    import torch
    from spd_gb300 import SDADER_Simulator
    kind, target = FULL_RUNS[args.workload]
    kw = workload_kwargs(args.workload, args.cells)
    dof, cells = dof_of(kw)
    t_setup = time.perf_counter()
    s = SDADER_Simulator(verbose=False, fma=args.build == "fma", **kw)
    t_setup = time.perf_counter() - t_setup
    stream = torch.cuda.current_stream()
    s._ctx.set_stream(stream.cuda_stream)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    import contextlib
    # the drivers' end-of-run line (the reference prints it) goes to stderr:
    # stdout carries the one JSON line
    with ClockSampler(0) as clk, contextlib.redirect_stdout(sys.stderr):
        e0.record(stream)
        if kind == "t_end":
            s.perform_time_evolution(target)
        else:
            s.perform_iterations(target)
        e1.record(stream)
        torch.cuda.synchronize()
    ms = e0.elapsed_time(e1)
    U = s.dm.U_sp
    out = {"metric": METRIC + " over a whole run", "value": dof * s.n_step / (ms / 1e3), "unit": UNIT,
           "n_gpus": 1, "higher_is_better": True, "dtype": "f64", "data": "synthetic", "build": args.build,
           "config": {"workload": WORKLOADS[args.workload], "cells": cells, "dof": dof, "run": {kind: target}},
           "steps": s.n_step, "t_final": s.time, "time_to_solution_s": ms / 1e3, "ms_per_step": ms / s.n_step,
           "setup_s": t_setup, "finite": bool(np.isfinite(U).all()),
           "troubled_subcells_last_step": float(s.dm.troubles.sum()) if s.update == "FV" and s.FB else None,
           "clocks": clk.summary()}
    s.close()
    print(json.dumps(out), flush=True)


def reference_arm(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    procs = os.cpu_count() or 1
    n_side = {"quadrant512": 64, "vortex32": 32, "sedov128": 12, "vortex512_sd": 64,
              "quadrant512_lhllc_moncen": 64}[args.workload]
    steps = max(1, args.steps)
    value, tmax = cpu_baseline(args.workload, n_side, steps, args.warmup, procs)
    kw = workload_kwargs(args.workload, n_side)
    sample = (f"{procs} independent processes, each {args.warmup}+{steps} steps of the same configuration at "
              f"{'x'.join(str(n) for n in kw['N'])} cells (the full grid needs ~9 GB and ~90 s per step per core)")
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus, "steps": steps,
            "warmup": args.warmup, "ms_per_step": tmax / steps * 1e3, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic", "impl": "reference",
            "config": {"workload": WORKLOADS[args.workload], "sample_cells": kw["N"]},
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": procs, "kind": "port", "sample": sample},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------------------
# multi-process bookkeeping (replicas: one process per GPU, no collective on
# the data path; the slowest rank's time defines the job's time)
# ---------------------------------------------------------------------------
def max_over_ranks(ms, dist, device):
    """The maximum of ``ms`` over all ranks (``dist`` None: single process)."""
    if dist is None:
        return float(ms)
    import torch
    t = torch.tensor([float(ms)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def whole_job_rate(units_per_rank_step, steps, world, ms):
    """Units processed by all ranks per second over the slowest rank's time."""
    return units_per_rank_step * steps * world / (ms / 1e3)


def shard_instances(work, world):
    """Independent ensemble instances split over ``world`` ranks (no
    collective on the data path): largest first, each to the rank with the
    least work so far.  Returns the instance indices of every rank."""
    load = [0] * world
    shards = [[] for _ in range(world)]
    for i in sorted(range(len(work)), key=lambda k: (-work[k], k)):
        r = min(range(world), key=lambda q: (load[q], q))
        shards[r].append(i)
        load[r] += work[i]
    return [sorted(s) for s in shards]


# ---------------------------------------------------------------------------
# the GPU arm
# ---------------------------------------------------------------------------
def ours(args):
    import numpy as np
    import torch
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    from spd_gb300 import SDADER_Simulator
    kw = workload_kwargs(args.workload, args.cells)
    dof, cells = dof_of(kw)
    s = SDADER_Simulator(verbose=False, fma=args.build == "fma", **kw)
    ctx = s._ctx
    stream = torch.cuda.current_stream()
    ctx.set_stream(stream.cuda_stream)
    # warm-up
    for _ in range(args.warmup):
        s.compute_dt()
        s.perform_update()
    torch.cuda.synchronize()
    launches0 = ctx.launch_count()
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    # the timed region: compute_dt + perform_update per step, launch by
    # launch, no per-kernel events (inputs are larger than L2: U_sp alone is
    # 134 MB at 512^2, a step touches several GB)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(local) as clk:
        e0.record(stream)
        for _ in range(args.steps):
            s.compute_dt()
            s.perform_update()
        e1.record(stream)
        torch.cuda.synchronize()
    ms = max_over_ranks(e0.elapsed_time(e1), dist, "cuda")
    if dist:
        dist.barrier()
    launches = ctx.launch_count() - launches0
    clocks = clk.summary()
    value = whole_job_rate(dof, args.steps, world, ms)

    # a separate pass with a CUDA-event pair around every launch (on the
    # library's stream) for the per-kernel split and the kernel roofline
    prof_steps = max(1, min(args.steps, 5))
    ctx.profile_report()
    ctx.profile(True)
    p0, p1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    p0.record(stream)
    for _ in range(prof_steps):
        s.compute_dt()
        s.perform_update()
    p1.record(stream)
    torch.cuda.synchronize()
    ctx.profile(False)
    prof = ctx.profile_report()
    prof_ms = p0.elapsed_time(p1)

    if args.lean:
        print(json.dumps({"metric": METRIC, "value": value, "unit": UNIT, "ms_per_step": ms / args.steps,
                          "build": args.build, "lean": True,
                          "kernels_ms": {k: round(v[1], 3) for k, v in prof.items()}}), flush=True)
        s.close()
        return
    # the same steps through perform_iterations' driver: one captured step
    # (CUDA graph) replayed per step, dt and time kept on the device
    s.time, _, _ = ctx.step(1, 0.0, 0, s.time)  # capture (untimed)
    torch.cuda.synchronize()
    g0, g1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    g0.record(stream)
    s.time, _, _ = ctx.step(args.steps, 0.0, 0, s.time)
    g1.record(stream)
    torch.cuda.synchronize()
    graph_ms = g0.elapsed_time(g1)
    graph_driver = {"ms_per_step": graph_ms / args.steps, "value": whole_job_rate(dof, args.steps, 1, graph_ms)}

    # end to end through the public API with host buffers
    shape_u = s._shape_of("U_sp")
    shape_w = s._shape_of("W_cv")
    U_host = torch.empty(int(np.prod(shape_u)), dtype=torch.float64, pin_memory=True).numpy().reshape(shape_u)
    W_host = torch.empty(int(np.prod(shape_w)), dtype=torch.float64, pin_memory=True).numpy().reshape(shape_w)
    U_host[...] = s.dm.U_sp
    W_host[...] = s.dm.W_cv
    out = torch.empty(int(np.prod(shape_u)), dtype=torch.float64, pin_memory=True).numpy().reshape(shape_u)
    e2e_steps = max(1, min(args.steps, 10))

    def e2e_step():
        s._ctx.upload("U_sp", U_host)
        s._ctx.upload("W_cv", W_host)
        s.compute_dt()
        s.perform_update()
        s._ctx.check(s._ctx.lib.spd_download(s._ctx.h, 0, out.ctypes.data_as(
            __import__("ctypes").POINTER(__import__("ctypes").c_double)), out.size), "download")

    e2e_step()  # untimed: first use of the transfer staging buffer
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        e2e_step()
    e2e_s = time.perf_counter() - t0
    e2e = {"value": dof * e2e_steps * world / e2e_s, "unit": UNIT,
           "h2d_bytes_per_step": int(U_host.nbytes + W_host.nbytes), "d2h_bytes_per_step": int(out.nbytes),
           "steps": e2e_steps}

    # roofline of the dominant kernel: the FP64 pipe binds (the step moves
    # ~1 KB of compulsory HBM traffic per cell and computes ~1e5 operations)
    fp64, fp64_clocks = None, None
    if rank == 0:
        try:
            with ClockSampler(local) as clk64:
                fp64 = fp64_peak_tflops()
            fp64_clocks = clk64.summary()
        except Exception:
            fp64 = None
    D, p = len(kw["N"]), kw["p"]
    m = p
    upd = kw.get("update", "SD")
    roof, issue, hbm = None, None, None
    kint = prof.get("k_interior")
    if kint:
        flops_step = interior_flops_per_cell_step(D, p, m, upd) * cells
        nlaunch = kint[0] / prof_steps
        per_launch_flops = flops_step / nlaunch
        avg_s = kint[1] / kint[0] / 1e3
        achieved = per_launch_flops / avg_s / 1e12
        ncu = NCU_K_INTERIOR.get((D, p, upd, args.build))
        roof = {"bound": "fp64", "kernel": "k_interior", "achieved": achieved,
                "peak": fp64, "unit": "TFLOP/s", "frac": (achieved / fp64) if fp64 else None,
                "peak_kind": "measured in this run: cuBLAS DGEMM 8192^3 FP64 (burst; no FP64 entry in "
                             "MEASURED_PEAKS.json)",
                "traffic": ncu["dram_bytes"] * cells / nlaunch if ncu else None,
                "traffic_kind": (f"ncu DRAM read+write per launch at {int(ncu['cells_captured'] ** 0.5)}^2 cells, "
                                 "scaled by the cell count") if ncu else None,
                "algorithmic_flops_per_launch": per_launch_flops,
                "algorithmic_flops_per_cell_step": interior_flops_per_cell_step(D, p, m, upd),
                "launches_per_step": nlaunch, "avg_launch_ms": avg_s * 1e3}
        if ncu and fp64:
            rate = ncu["fp64_inst"] * cells * prof_steps / (kint[1] / 1e3)
            peak_issue = fp64 * 1e12 / 2.0
            issue = {"kernel": "k_interior", "fp64_instructions_per_cell_step": ncu["fp64_inst"],
                     "achieved_g_inst_per_s": rate / 1e9, "peak_g_inst_per_s": peak_issue / 1e9,
                     "frac": rate / peak_issue,
                     "meaning": "FP64 pipe occupancy: executed DADD+DMUL+DFMA (each 1) against cuBLAS DGEMM's "
                                "DFMA issue rate; not a flop fraction"}
    peak_gbs, peak_kind = measured_peaks()
    hb = compulsory_bytes_per_cell_step(D, p) * cells / (ms / args.steps / 1e3) / 1e9
    hbm = {"compulsory_bytes_per_cell_step": compulsory_bytes_per_cell_step(D, p), "achieved": hb,
           "peak": peak_gbs, "unit": "GB/s", "frac": hb / peak_gbs, "peak_kind": peak_kind}
    total_kernel_ms = sum(v[1] for v in prof.values())
    fma = None
    if rank == 0 and world == 1 and not args.no_fma and args.build == "ieee":
        fma = fma_build_section(args, kw, s, stream, dof, cells, fp64, ms / args.steps)
    line = None
    if rank == 0:
        cpu = None
        parity = None
        if world == 1 and not args.no_cpu_baseline:
            sample_n = 128 if len(kw["N"]) == 2 else 16
            v, tmax, U_oracle = cpu_baseline(args.workload, sample_n, 1, 0, 1, want_state=True)
            parity = sample_parity(args.workload, sample_n, U_oracle)
            cpu = {"value": v, "unit": UNIT, "cores": 1, "kind": "port",
                   "sample": f"1 step of the same configuration at {'x'.join([str(sample_n)] * len(kw['N']))} cells on one core "
                             "(CPU restatement of the reference's NumPy path)"}
        line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True, "build": args.build,
                "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
                "config": {"workload": WORKLOADS[args.workload] + (f" (reduced to {args.cells} cells per side)"
                                                                   if args.cells else ""),
                           "cells": cells, "dof": dof,
                           "parallelism": "replicas" if world > 1 else "single",
                           "l2": "inputs larger than L2: U_sp alone is "
                                 f"{dof * (D + 2) * 8 / 1e6:.0f} MB, step working set several GB"},
                "roofline": roof,
                "fp64_issue": issue,
                "fma_build": fma,
                "hbm_compulsory": hbm,
                "fp64_gemm_peak_tflops": fp64, "fp64_gemm_clocks": fp64_clocks,
                "cpu_baseline": cpu, "parity_vs_oracle": parity,
                "vortex_t1": vortex_t1_error() if world == 1 else None,
                "other_configs": other_configs(args) if world == 1 and not args.cells else None,
                "graph_driver": graph_driver,
                "e2e": e2e, "gpu_launches": launches,
                "clocks": clocks,
                "profiled_pass": {"steps": prof_steps, "ms_per_step": prof_ms / prof_steps,
                                  "kernels_ms": {k: round(v[1], 3)
                                                 for k, v in sorted(prof.items(), key=lambda kv: -kv[1][1])},
                                  "kernel_share_of_step": total_kernel_ms / prof_ms if prof_ms else None}}
        print(json.dumps(line), flush=True)
    s.close()
    if dist:
        dist.destroy_process_group()


def fma_build_section(args, kw, s_ieee, stream, dof, cells, fp64, ieee_ms_step):
    """The same workload on the library built with fused multiply-adds
    (SDADER_Simulator(fma=True)): its step time (timed like the headline),
    its k_interior flop-basis roofline, and its deviation from the product
    build (bit-identical to the reference) over 10 steps from the same
    initial state: normwise relative difference of U_sp per variable and the
    steps whose trouble masks differ."""
    import numpy as np
    import torch
    from spd_gb300 import SDADER_Simulator
    try:
        f = SDADER_Simulator(verbose=False, fma=True, **kw)
    except ImportError as err:
        return {"unavailable": str(err)}
    ctx = f._ctx
    ctx.set_stream(stream.cuda_stream)
    for _ in range(args.warmup):
        f.compute_dt()
        f.perform_update()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.steps):
        f.compute_dt()
        f.perform_update()
    e1.record(stream)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / args.steps
    prof_steps = max(1, min(args.steps, 5))
    ctx.profile_report()
    ctx.profile(True)
    for _ in range(prof_steps):
        f.compute_dt()
        f.perform_update()
    torch.cuda.synchronize()
    ctx.profile(False)
    prof = ctx.profile_report()
    D, p = len(kw["N"]), kw["p"]
    kint = prof.get("k_interior")
    roof = None
    if kint:
        achieved = interior_flops_per_cell_step(D, p, p, kw.get("update", "SD")) * cells * prof_steps / (
            kint[1] / 1e3) / 1e12
        roof = {"kernel": "k_interior", "achieved": achieved, "peak": fp64, "unit": "TFLOP/s",
                "frac": achieved / fp64 if fp64 else None, "avg_launch_ms": kint[1] / kint[0]}
        ncu = NCU_K_INTERIOR.get((D, p, kw.get("update", "SD"), "fma"))
        if ncu and fp64:
            rate = ncu["fp64_inst"] * cells * prof_steps / (kint[1] / 1e3)
            roof["fp64_issue_frac"] = rate / (fp64 * 1e12 / 2.0)
            roof["fp64_instructions_per_cell_step"] = ncu["fp64_inst"]
    f.close()
    # deviation from the product build over 10 steps from one initial state
    # (fresh simulators: the FV boundary buffers start from the initial
    # condition in both)
    a = SDADER_Simulator(verbose=False, **kw)
    f = SDADER_Simulator(verbose=False, fma=True, **kw)
    limited = a.update == "FV" and a.FB
    flips, devs = 0, {}
    for k in range(10):
        a.compute_dt()
        f.compute_dt()
        a.perform_update()
        f.perform_update()
        if limited and not np.array_equal(a.dm.troubles, f.dm.troubles):
            flips += 1
        if k in (0, 9):
            Ua, Uf = a.dm.U_sp, f.dm.U_sp
            devs[f"after_{k + 1}_steps"] = max(float(np.max(np.abs(Uf[v] - Ua[v])) / np.max(np.abs(Ua[v])))
                                               for v in range(Ua.shape[0]))
    a.close()
    f.close()
    return {"value": dof / (ms / 1e3), "unit": UNIT, "ms_per_step": ms, "speedup_over_product_build": ieee_ms_step / ms,
            "roofline": roof, "normwise_rel_dev_U_sp": devs, "steps_with_trouble_mask_differences": flips,
            "kernels_ms": {k: round(v[1], 3) for k, v in sorted(prof.items(), key=lambda kv: -kv[1][1])[:8]}}


def ensemble_arm(args):
    """Batched ensemble vs the plain per-instance loop on the same instances.
    Under torchrun the instances are sharded over the ranks (balanced by
    DOF, no collective on the data path; strong scaling: the ensemble is
    fixed); each rank advances its share, the slowest rank's time counts."""
    import numpy as np
    import torch
    from spd_gb300 import SDADER_Ensemble, SDADER_Simulator
    from spd_gb300.initial_conditions import kelvin_helmholtz
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    rng = np.random.default_rng(2026)
    small = args.workload == "kh_ensemble_small"
    choices = [16, 24, 32, 48, 64] if small else [64, 128, 192, 256, 384, 512]
    sides = [int(x) for x in rng.choice(choices, size=args.instances)]
    mine = shard_instances([n * n for n in sides], world)[rank]

    def make(i, n):
        return SDADER_Simulator(p=3, N=(n, n), init_fct=kelvin_helmholtz(n, seed=1000 + i), update="FV", FB=True,
                                riemann_solver_sd="hllc", riemann_solver_fv="hllc",
                                BC=(("periodic", "periodic"),) * 2, verbose=False)

    def timed(fn):
        """fn's wall time on this rank between synchronised starts, max over ranks (s)."""
        torch.cuda.synchronize()
        if dist:
            dist.barrier()
        t0 = time.perf_counter()
        fn()
        torch.cuda.synchronize()
        return max_over_ranks((time.perf_counter() - t0) * 1e3, dist, "cuda") / 1e3

    sims = [make(i, sides[i]) for i in mine]
    dof = sum(n * n * 16 for n in sides)

    def plain_loop(nsteps):
        # plain per-instance loop (compute_dt + perform_update per instance and step)
        for sm in sims:
            for _ in range(nsteps):
                sm.compute_dt()
                sm.perform_update()

    plain_loop(args.warmup)
    with ClockSampler(int(os.environ.get("LOCAL_RANK", "0"))) as clk_plain:
        plain_s = timed(lambda: plain_loop(args.steps))
    ens, tuning = None, None
    if sims:
        if args.ensemble_form == "auto":
            ens = SDADER_Ensemble(sims)
            tuning = ens.autotune(streams=(1, 4, 16), cpbs=(32, 64), probe_launches=1)
        else:
            ens = SDADER_Ensemble(sims, nstreams=16, packed=args.ensemble_form == "packed")
            tuning = {"form": args.ensemble_form, "streams": None if args.ensemble_form == "packed" else 16,
                      "cells_per_block": ens.cells_per_block()[0][0], "graph_nodes_per_step": ens.graph_nodes()}
        ens.perform_iterations(args.warmup)
    with ClockSampler(int(os.environ.get("LOCAL_RANK", "0"))) as clk_batched:
        batched_s = timed(lambda: ens.perform_iterations(args.steps) if ens else None)
    plain = dof * args.steps / plain_s
    batched = dof * args.steps / batched_s
    if rank == 0:
        line = {"metric": METRIC + "; batched/plain speedup", "value": batched, "unit": UNIT, "n_gpus": world,
                "steps": args.steps, "warmup": args.warmup, "ms_per_step": batched_s / args.steps * 1e3,
                "higher_is_better": True, "scaling": "strong" if world > 1 else "weak", "vs_baseline": None,
                "dtype": "f64", "data": "synthetic",
                "config": {"workload": WORKLOADS[args.workload], "instances": len(sides), "sides": sides,
                           "dof_per_ensemble_step": dof,
                           "parallelism": f"instances sharded over {world} GPUs" if world > 1 else "1 GPU"},
                "plain_loop_value": plain, "plain_loop_ms_per_step": plain_s / args.steps * 1e3,
                "batched_over_plain": batched / plain, "autotune": tuning,
                "clocks": clk_batched.summary(), "plain_loop_clocks": clk_plain.summary()}
        print(json.dumps(line), flush=True)
    if ens:
        ens.close()
    for sm in sims:
        sm.close()
    if dist:
        dist.destroy_process_group()


def adjoint_arm(args):
    """Forward and backward (adjoint) time of the KH gradient; the headline
    value is gradients/s, with the backward/forward time ratio beside it."""
    import numpy as np
    import torch
    from spd_gb300 import SDADER_Simulator
    from spd_gb300.adjoint import AdjointRunner
    from spd_gb300.initial_conditions import kelvin_helmholtz
    n = args.cells or 256
    nsteps = args.adj_steps

    def make(seed=7):
        return SDADER_Simulator(p=3, N=(n, n), init_fct=kelvin_helmholtz(n, seed=seed), update="FV", FB=True,
                                riemann_solver_sd="hllc", riemann_solver_fv="hllc",
                                BC=(("periodic", "periodic"),) * 2, verbose=False)

    s = make()
    U0 = torch.tensor(s.dm.U_sp, device="cuda")
    shape = tuple(U0.shape)
    rng = np.random.default_rng(2027)
    Ut = U0.clone()
    Ut[0] = U0[0] * (1.0 + 1e-2 * torch.tensor(rng.standard_normal(shape[1:]), device="cuda"))
    target = AdjointRunner(s, nsteps).forward(Ut)[0].clone()

    # plain forward (the step loop without checkpoints) for the cost ratio
    s.dm.U_sp = U0.cpu().numpy()
    s._ctx.end_sim()
    for _ in range(args.warmup):
        s.compute_dt()
        s.perform_update()
    s.dm.U_sp = U0.cpu().numpy()
    s._ctx.end_sim()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    s.time, done, _ = s._ctx.step(nsteps, 0.0, 0, s.time)
    torch.cuda.synchronize()
    plain_s = time.perf_counter() - t0
    results = []
    with ClockSampler() as clk:
        for rep in range(max(1, args.steps)):
            r = AdjointRunner(s, nsteps)
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            y = r.forward(U0)
            res = y[0] - target
            J = float((res * res).sum())
            gy = torch.zeros_like(y)
            gy[0] = 2.0 * res
            torch.cuda.synchronize()
            t1 = time.perf_counter()
            g = r.backward(gy)
            torch.cuda.synchronize()
            t2 = time.perf_counter()
            results.append((t1 - t0, t2 - t1))
    fwd_s = min(a for a, _ in results)
    bwd_s = min(b for _, b in results)
    grad_rho = g[0]
    # per-kernel device time of one more forward + backward (CUDA events)
    s._ctx.profile(True)
    r = AdjointRunner(s, nsteps)
    y = r.forward(U0)
    fwd_prof = s._ctx.profile_report()
    r.backward(gy)
    bwd_prof = s._ctx.profile_report()
    s._ctx.profile(False)
    top = sorted(bwd_prof.items(), key=lambda kv: -kv[1][1])[:10]
    line = {"metric": "gradients/s (KH 256^2, p=3, 200 steps, FP64 adjoint)", "value": 1.0 / (fwd_s + bwd_s),
            "unit": "gradients/s", "n_gpus": 1, "steps": len(results), "warmup": args.warmup,
            "ms_per_step": (fwd_s + bwd_s) * 1e3, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": WORKLOADS["kh_adjoint"], "cells": [n, n], "time_steps": nsteps,
                       "checkpoint_every": r.k},
            "forward_plain_s": plain_s, "forward_with_checkpoints_s": fwd_s, "backward_s": bwd_s,
            "backward_over_forward": bwd_s / plain_s, "J": J,
            "grad_rho_norm": float(torch.linalg.vector_norm(grad_rho)), "clocks": clk.summary(),
            "forward_kernels_ms": round(sum(v[1] for v in fwd_prof.values()), 3),
            "backward_kernels_ms": round(sum(v[1] for v in bwd_prof.values()), 3),
            "backward_top_kernels_ms": {k: [v[0], round(v[1], 3)] for k, v in top}}
    if args.fd_dirs:
        line["fd_check"] = adjoint_fd_check(s, U0, target, r.dts, g, args.fd_dirs)
    s.close()
    if args.batch > 1:
        line["batch"] = adjoint_batch(args, make_batch=lambda i: make(seed=100 + i), n=n, nsteps=nsteps)
    print(json.dumps(line), flush=True)


def adjoint_fd_check(s, U0, target, dts, g, ndirs, eps=1e-6, seed=2028):
    """Central differences of J along seeded density-only directions
    (entrywise relative to the density) against the adjoint gradient.  The
    perturbed runs replay the forward's dts and every decision (affected
    faces, Riemann-solver and limiter branches) from decision tapes, so
    both sides see the same frozen-decision map."""
    import numpy as np
    import torch
    ctx = s._ctx
    nsteps = len(dts)
    shape = tuple(U0.shape)
    count = U0.numel()
    ctx.tape_enable(nsteps)

    def put(x):
        x = x.contiguous()
        torch.cuda.synchronize()
        ctx.upload_ptr("U_sp", x.data_ptr(), count)

    def run(mode):
        for j in range(nsteps):
            ctx.tape_step(j, dts[j], mode)
        y = torch.empty(shape, dtype=torch.float64, device="cuda")
        torch.cuda.synchronize()
        ctx.download_ptr("U_sp", y.data_ptr(), count)
        res = y[0] - target
        return float((res * res).sum())

    put(U0)
    J0 = run(1)
    put(U0)
    J0r = run(2)
    rng = np.random.default_rng(seed)
    errs = []
    t0 = time.perf_counter()
    for _ in range(ndirs):
        v = torch.zeros_like(U0)
        v[0] = torch.tensor(rng.standard_normal(shape[1:]), device="cuda") * U0[0].abs()
        put(U0 + eps * v)
        Jp = run(2)
        put(U0 - eps * v)
        Jm = run(2)
        fd = (Jp - Jm) / (2 * eps)
        ad = float((g * v).sum())
        errs.append(abs(fd - ad) / abs(ad))
    return {"directions": ndirs, "eps_relative": eps, "replay_reproduces_forward": J0 == J0r,
            "median_rel_err": float(np.median(errs)), "max_rel_err": float(np.max(errs)),
            "rel_errs": [float("%.3e" % e) for e in errs], "seconds": time.perf_counter() - t0}


def adjoint_batch(args, make_batch, n, nsteps):
    """B seeded instances (own targets), each gradient on its own context and
    stream, driven by ``spd_gb300.adjoint.AdjointBatch`` (one host thread per
    instance)."""
    import numpy as np
    import torch
    from spd_gb300.adjoint import AdjointBatch, AdjointRunner
    B = args.batch
    sims = [make_batch(i) for i in range(B)]
    U0s = [torch.tensor(sm.dm.U_sp, device="cuda") for sm in sims]
    targets = []
    for i, sm in enumerate(sims):
        rng = np.random.default_rng(3000 + i)
        Ut = U0s[i].clone()
        Ut[0] = U0s[i][0] * (1.0 + 1e-2 * torch.tensor(rng.standard_normal(tuple(Ut.shape[1:])), device="cuda"))
        targets.append(AdjointRunner(sm, nsteps).forward(Ut)[0].clone())
    torch.cuda.synchronize()

    # a record slot holds ~1 GB at 256^2 against 34 MB per U_sp checkpoint:
    # 16 concurrent instances keep 4 slots each (checkpoints every 4 steps)
    every = 4

    def loss_grad(i, y):
        gy = torch.zeros_like(y)
        gy[0] = 2.0 * (y[0] - targets[i])
        return gy

    batch = AdjointBatch(sims, nsteps, checkpoint_every=every)
    t0 = time.perf_counter()
    _, grads = batch.gradients(U0s, loss_grad)
    torch.cuda.synchronize()
    wall = time.perf_counter() - t0
    norms = [float(torch.linalg.vector_norm(g[0])) for g in grads]
    for sm in sims:
        sm.close()
    return {"instances": B, "wall_s": wall, "gradients_per_s": B / wall, "checkpoint_every": every,
            "grad_rho_norms": norms}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="quadrant512", choices=sorted(WORKLOADS))
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-fma", action="store_true", help="skip the fused multiply-add build's section")
    ap.add_argument("--lean", action="store_true",
                    help="only the timed and profiled passes (no graph driver, end-to-end, DGEMM, vortex, CPU "
                         "baseline or fma sections): a short launch sequence for profilers")
    ap.add_argument("--build", default="ieee", choices=["ieee", "fma"],
                    help="library of the headline simulator: the product (bit-identical to the reference) or the "
                         "fused multiply-add build")
    ap.add_argument("--instances", type=int, default=64, help="ensemble size (kh_ensemble)")
    ap.add_argument("--ensemble-form", default="auto", choices=["auto", "packed", "streams"],
                    help="batched form (kh_ensemble): autotuned, or fixed without tuning")
    ap.add_argument("--cells", type=int, default=None,
                    help="cells per direction (a smaller case of the workload, for profiling)")
    ap.add_argument("--adj-steps", type=int, default=200, help="time steps of the differentiated run (kh_adjoint)")
    ap.add_argument("--fd-dirs", type=int, default=0, help="central-difference directions to check (kh_adjoint)")
    ap.add_argument("--batch", type=int, default=1, help="seeded instances run concurrently (kh_adjoint)")
    ap.add_argument("--full-run", action="store_true",
                    help="the workload's whole run as its configuration specifies (t_end or step count) through "
                         "perform_time_evolution / perform_iterations")
    args = ap.parse_args()
    if args.impl == "reference":
        reference_arm(args)
    elif args.workload == "kh_adjoint" and int(os.environ.get("RANK", "0")):
        return  # the adjoint workload runs on one GPU: under torchrun only rank 0 runs it
    elif args.workload in ("kh_ensemble", "kh_ensemble_small"):
        from spd_gb300.build import build
        if int(os.environ.get("LOCAL_RANK", "0")) == 0:
            build()
        if args.workload == "kh_ensemble_small" and args.instances == 64:
            args.instances = 256
        ensemble_arm(args)
    elif args.workload == "kh_adjoint":
        from spd_gb300.build import build
        build()
        adjoint_arm(args)
    elif args.full_run:
        from spd_gb300.build import build
        build()
        full_run_arm(args)
    else:
        from spd_gb300.build import build
        if int(os.environ.get("LOCAL_RANK", "0")) == 0:
            build()
        ours(args)


if __name__ == "__main__":
    main()
