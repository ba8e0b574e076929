"""Batched ensembles of independent SD-ADER problems (no reference
counterpart).

``SDADER_Ensemble`` advances many ``SDADER_Simulator`` instances of
different grid sizes together, each with its own CFL dt, in one of two
forms (C ABI: ``spd_ensemble_*``):

* ``packed=True`` (default): every stage of the step (CFL reduction, predictor
  kernels, FV update, trouble detection, fallback) is ONE launch over all
  instances; a per-instance block-offset table maps each thread block to its
  instance and to its block within that instance.  A whole ensemble step is
  one CUDA graph of ~130 launches (2D, p=3, limiting), however many
  instances there are.
* ``packed=False``: the per-instance step sequences are recorded into one
  CUDA graph whose branches run on ``nstreams`` streams.

``autotune`` picks the form, the number of streams and the cells per block
of the predictor's fused kernel by timing real ensemble steps.  Every
instance produces the same bits as stepping it alone.
"""
from __future__ import annotations

import ctypes
import time

from . import _lib


class SDADER_Ensemble:
    def __init__(self, simulators, nstreams: int = 8, steps_per_launch: int = 1, packed: bool = True):
        self.sims = list(simulators)
        if not self.sims:
            raise ValueError("empty ensemble")
        variants = {getattr(s._ctx, "variant", "ieee") for s in self.sims}
        if len(variants) > 1:
            raise ValueError("an ensemble needs every instance built from one library (all fma=True or none)")
        self.lib = _lib.load(variants.pop())
        self._declare()
        self.nstreams = nstreams
        self.steps_per_launch = steps_per_launch
        self.packed = packed
        self.tuning = None
        self._ens = None
        self._build()

    def _declare(self):
        lib = self.lib
        vp = ctypes.c_void_p
        lib.spd_ensemble_create.argtypes = [ctypes.POINTER(vp), ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                            ctypes.POINTER(vp)]
        lib.spd_ensemble_create_packed.argtypes = [ctypes.POINTER(vp), ctypes.c_int, ctypes.c_int,
                                                   ctypes.POINTER(vp)]
        lib.spd_ensemble_graph_nodes.argtypes = [vp, ctypes.POINTER(ctypes.c_longlong)]
        lib.spd_ensemble_step.argtypes = [vp, ctypes.c_int]
        lib.spd_ensemble_synchronize.argtypes = [vp]
        lib.spd_ensemble_time.argtypes = [vp, ctypes.c_int, ctypes.POINTER(ctypes.c_double)]
        lib.spd_ensemble_set_time.argtypes = [vp, ctypes.c_int, ctypes.c_double]
        lib.spd_ensemble_destroy.argtypes = [vp]
        lib.spd_ensemble_last_error.argtypes = [vp]
        lib.spd_ensemble_last_error.restype = ctypes.c_char_p
        lib.spd_set_cells_per_block.argtypes = [vp, ctypes.c_int]
        lib.spd_get_cells_per_block.argtypes = [vp, ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_int)]

    def _check(self, rc, what):
        if rc != 0:
            msg = self.lib.spd_ensemble_last_error(self._ens) if self._ens else b""
            raise _lib.SpdError(f"{what}: status {rc}: {msg.decode() if msg else ''}")

    def _build(self):
        self._close()
        arr = (ctypes.c_void_p * len(self.sims))(*[s._ctx.h.value for s in self.sims])
        h = ctypes.c_void_p()
        if self.packed:
            rc = self.lib.spd_ensemble_create_packed(arr, len(self.sims), self.steps_per_launch, ctypes.byref(h))
        else:
            rc = self.lib.spd_ensemble_create(arr, len(self.sims), self.nstreams, self.steps_per_launch,
                                              ctypes.byref(h))
        if rc != 0:
            msg = self.lib.spd_ensemble_last_error(None)
            hint = ("; the packed form needs one dimension, degree, option set and cells per block "
                    "(packed=False advances instances that differ)") if self.packed else ""
            raise _lib.SpdError(f"ensemble create failed with status {rc}: {msg.decode() if msg else ''}{hint}")
        self._ens = h

    def graph_nodes(self) -> int:
        """Nodes (launches, zero-fills, stream joins) of one ensemble step's
        CUDA graph."""
        n = ctypes.c_longlong()
        self._check(self.lib.spd_ensemble_graph_nodes(self._ens, ctypes.byref(n)), "graph_nodes")
        return n.value

    def _close(self):
        if self._ens is not None and self._ens.value:
            self.lib.spd_ensemble_destroy(self._ens)
        self._ens = None

    def _push_times(self):
        """Start the device time accumulators from the instances' times, so
        they add the dts exactly as the host loop does."""
        for i, s in enumerate(self.sims):
            self._check(self.lib.spd_ensemble_set_time(self._ens, i, float(s.time)), "set_time")

    def _sync_times(self, steps):
        self._check(self.lib.spd_ensemble_synchronize(self._ens), "synchronize")
        for i, s in enumerate(self.sims):
            t = ctypes.c_double()
            self._check(self.lib.spd_ensemble_time(self._ens, i, ctypes.byref(t)), "time")
            s.time = t.value
            s.n_step += steps

    def cells_per_block(self):
        out = []
        for s in self.sims:
            c, m = ctypes.c_int(), ctypes.c_int()
            self.lib.spd_get_cells_per_block(s._ctx.h, ctypes.byref(c), ctypes.byref(m))
            out.append((c.value, m.value))
        return out

    def set_cells_per_block(self, cpb: int):
        for s in self.sims:
            c, m = ctypes.c_int(), ctypes.c_int()
            self.lib.spd_get_cells_per_block(s._ctx.h, ctypes.byref(c), ctypes.byref(m))
            self.lib.spd_set_cells_per_block(s._ctx.h, min(cpb, m.value))

    def perform_iterations(self, n_step: int) -> None:
        """Advance every instance n_step steps (each with its own dt)."""
        if n_step % self.steps_per_launch:
            raise ValueError("n_step must be a multiple of steps_per_launch")
        launches = n_step // self.steps_per_launch
        self._push_times()
        self._check(self.lib.spd_ensemble_step(self._ens, launches), "step")
        self._sync_times(n_step)

    def autotune(self, streams=(1, 2, 4, 8, 16, 32), cpbs=(16, 32, 64), probe_launches: int = 2,
                 packed=(True, False)):
        """Time real ensemble steps for every candidate -- the packed form
        and the stream form with each number of streams, at each cells per
        block -- and keep the fastest.  The probe steps advance the
        instances and count as steps.  A candidate whose ensemble cannot be
        created (the packed form for instances that differ in dimension,
        degree or options) is skipped and listed in ``tuning["skipped"]``;
        if no candidate builds, the form in use before the call is rebuilt
        and the error is raised."""
        prev = (self.packed, self.nstreams, self.cells_per_block())
        results, skipped = {}, {}
        forms = [("packed", 0)] if True in packed else []
        if False in packed:
            forms += [("streams", ns) for ns in streams]
        for cpb in cpbs:
            self.set_cells_per_block(cpb)
            for form, ns in forms:
                self.packed = form == "packed"
                self.nstreams = ns or self.nstreams
                try:
                    self._build()
                except _lib.SpdError as err:
                    skipped[(form, ns, cpb)] = str(err)
                    continue
                self._push_times()
                self._check(self.lib.spd_ensemble_step(self._ens, 1), "warm-up")
                self._check(self.lib.spd_ensemble_synchronize(self._ens), "synchronize")
                t0 = time.perf_counter()
                self._check(self.lib.spd_ensemble_step(self._ens, probe_launches), "probe")
                self._check(self.lib.spd_ensemble_synchronize(self._ens), "synchronize")
                results[(form, ns, cpb)] = (time.perf_counter() - t0) / probe_launches
                self._sync_times((1 + probe_launches) * self.steps_per_launch)

        def label(k):
            return f"packed x{k[2]}" if k[0] == "packed" else f"{k[1]} streams x{k[2]}"

        if not results:
            self.packed, self.nstreams = prev[0], prev[1]
            for s, (c, _) in zip(self.sims, prev[2]):
                self.lib.spd_set_cells_per_block(s._ctx.h, c)
            self._build()
            raise _lib.SpdError("autotune: no candidate ensemble could be created: "
                                + "; ".join(f"{label(k)}: {v}" for k, v in skipped.items()))
        best = min(results, key=results.get)
        form, ns, cpb = best
        self.packed = form == "packed"
        self.nstreams = ns or self.nstreams
        self.set_cells_per_block(cpb)
        self._build()
        self.tuning = {"form": form, "streams": ns if form == "streams" else None, "cells_per_block": cpb,
                       "seconds_per_step": results[best] / self.steps_per_launch,
                       "graph_nodes_per_step": self.graph_nodes() // self.steps_per_launch,
                       "candidates": {label(k): v for k, v in sorted(results.items(), key=lambda kv: kv[1])},
                       "skipped": {label(k): v for k, v in skipped.items()}}
        return self.tuning

    def close(self):
        self._close()

    def __del__(self):
        try:
            self._close()
        except Exception:
            pass
