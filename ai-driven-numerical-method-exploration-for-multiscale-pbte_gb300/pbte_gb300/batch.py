"""Several solves at once on one GPU.

Every solve of a batch runs on its own CUDA stream, driven by its own host
thread, so the GPU overlaps their kernels: one solve's latency-bound
wavefront sweep (a block per in-plane velocity, far from filling 152 SMs
with work) shares the SMs with another's sweep, moments and Krylov kernels,
and one solve's host round trip per Arnoldi column hides behind another's
device work.  The solves' operators, iterates and Krylov bases stay
resident between runs (graphs are captured once, by :meth:`BatchSolver.prepare`,
because a capture synchronises the whole device).

Each result is the one the case gives alone: the solves share no buffers,
and every kernel's arithmetic is independent of what else runs.
"""
from __future__ import annotations

import ctypes
import threading
import time

import numpy as np
import torch

from .device import bury, device_lock, empty_graveyard
from .krylov import ArnoldiGraphs
from .solver import RunRecord, Solver

__all__ = ["BatchSolver", "LockstepBatch", "tune_batch_shape"]


class BatchSolver:
    """Run a list of :class:`Solver` objects concurrently.

    ``ring_shape`` (groups, threads per group) sets the sweep's block shape
    for batched runs: four groups of 64 let two sweep blocks share an SM."""

    def __init__(self, solvers: list[Solver], ring_shape: tuple[int, int] | None = (4, 64)):
        if not solvers:
            raise ValueError("empty batch")
        self.solvers = list(solvers)
        dev = self.solvers[0].device
        if any(s.device != dev for s in self.solvers):
            raise ValueError("all solves of a batch run on one device")
        self.device = dev
        self.streams = [torch.cuda.Stream(device=dev) for _ in self.solvers]
        if ring_shape is not None:
            for s in self.solvers:
                s.ctx.set_groups(*ring_shape)
        self.prepared = False
        self.wall_clock = 0.0

    def prepare(self) -> list[RunRecord]:
        """One solve of each case alone, then every Krylov column graph of
        each case captured, so no capture happens during a batched run."""
        recs = []
        for s, st in zip(self.solvers, self.streams):
            with torch.cuda.stream(st):
                s.reset()
                recs.append(s.run())
            for entry in s.__dict__.get("_krylov_cache", {}).values():
                obj = entry[2]
                if isinstance(obj, ArnoldiGraphs):
                    obj.capture_all()
        torch.cuda.synchronize(self.device)
        self.prepared = True
        return recs

    def run(self, reset: bool = True) -> list[RunRecord]:
        """Solve every case (from the zero state when ``reset``); returns the
        records in the order of the solvers."""
        if not self.prepared:
            self.prepare()
        n = len(self.solvers)
        results: list[RunRecord | None] = [None] * n
        errors: list[BaseException | None] = [None] * n

        def work(i: int) -> None:
            try:
                with torch.cuda.stream(self.streams[i]):
                    if reset:
                        self.solvers[i].reset()
                    results[i] = self.solvers[i].run()
            except BaseException as e:   # re-raised on the calling thread
                errors[i] = e

        torch.cuda.synchronize(self.device)
        t0 = time.perf_counter()
        threads = [threading.Thread(target=work, args=(i,), daemon=True) for i in range(n)]
        for t in threads:
            t.start()
        for t in threads:
            t.join()
        torch.cuda.synchronize(self.device)
        self.wall_clock = time.perf_counter() - t0
        for e in errors:
            if e is not None:
                raise e
        return results   # type: ignore[return-value]


class LockstepBatch:
    """Mixed-precision solves of many uneven cases advanced together, every
    inner FP32 product of all of them swept in ONE launch per DG order.

    Each case runs the defect correction of :func:`pbte_gb300.mixed.run_mixed`
    (FP64 defects; one inner GMRES cycle per outer step on FP32 products --
    source-iteration steps for CIS/GMRES cases, GSIS steps for GSIS cases).
    The cases' outer steps go in lockstep (:meth:`step`): all FP64 defects
    (concurrently, on side streams), then the inner cycles column by column,
    where column j of every case is [its moment sources] + one batched sweep
    (``pbte_sweep_batch_run``: the blocks are the distinct velocities of all
    cases of an order) + [its epilogue or GSIS chain, CGS2, rotation, next
    basis vector, on a side stream].  A case whose cycle has stopped (its
    device stop state) skips the rest of the cycle, and one that has
    converged skips everything; the host checks the states once per chunk of
    columns.  With ``use_graphs`` a chunk of all cases is one CUDA graph.
    Cases can join between steps (:meth:`add`) and leave when done
    (``step(remove_finished=True)``): continuous batching for a server.

    Each case's arithmetic is the one it has alone (the batched sweep gives
    the single sweep's bits), so the results are the solo results.
    ``shape = (groups, threads per group)`` is the batched sweep's block
    shape, the autotuner's knob (:func:`tune_batch_shape`)."""

    CHUNK = 10

    def __init__(self, solvers: list[Solver] = (), shape: tuple[int, int] = (4, 128), use_graphs: bool = True,
                 opts=None, lanes: int = 16, device=None):
        from .mixed import MixedOptions

        solvers = list(solvers)
        self.device = solvers[0].device if solvers else torch.device(device or "cuda")
        self.opts = opts or MixedOptions()
        self.use_graphs = use_graphs
        self.shape = shape
        self.cases = []
        self.handle = None
        self._dirty = True
        self.graphs = {}
        self.stream = torch.cuda.Stream(device=self.device)
        self.lanes = [torch.cuda.Stream(device=self.device) for _ in range(max(1, lanes))]
        self.wall_clock = 0.0
        for s in solvers:
            self.add(s)

    @property
    def solvers(self) -> list[Solver]:
        return [k["s"] for k in self.cases]

    def add(self, s: Solver) -> dict:
        """A mixed-precision solver joins the batch; its solve starts from
        zero at the next :meth:`step`."""
        from .krylov import FixedPointOperator, basis_cap, cached

        if s.device != self.device:
            raise ValueError("all solves of a batch run on one device")
        if s.precision != "mixed":
            raise ValueError("a lockstep batch runs mixed-precision solves")
        c = s.case
        if s.acc is not None:
            from .gsis import GsisFixedPoint
            op64 = cached(s, "gsis64", lambda: GsisFixedPoint(s, "fp64"))
            op32 = cached(s, "gsis32h", lambda: GsisFixedPoint(s, "fp32", homogeneous=True))
        else:
            op64 = cached(s, "fp64", lambda: FixedPointOperator(s, "fp64"))
            op32 = cached(s, "fp32h", lambda: FixedPointOperator(s, "fp32", homogeneous=True, integrals=False))
        cap = basis_cap(c, op64.n)
        bdt = torch.float32 if c.performance.inner_basis == "fp32" else torch.float64
        ar = cached(s, ("arnoldi_inner", cap, bdt, False), lambda: ArnoldiGraphs(op32, None, cap, dtype=bdt))
        ar._cycle_buffers()
        k = {"s": s, "op64": op64, "op32": op32, "ar": ar, "cap": cap, "fresh": True, "done": False,
             "converged": False}
        self.cases.append(k)
        self._dirty = True
        return k

    def _rebuild(self) -> None:
        """The batched sweep's case table for the current cases (and no
        captured chunk: they hold the old membership)."""
        from . import _lib
        bury(*self.graphs.values())
        self.graphs = {}
        if self.handle is not None and self.handle.value:
            _lib.lib().pbte_sweep_batch_destroy(self.handle)
            self.handle = None
        if self.cases:
            items = (_lib.BatchItem * len(self.cases))(*[k["op32"].batch_item(k["ar"].state) for k in self.cases])
            h = ctypes.c_void_p()
            _lib.check(_lib.lib().pbte_sweep_batch_create(len(self.cases), items, int(self.shape[0]),
                                                          int(self.shape[1]), ctypes.byref(h)), "sweep_batch_create")
            self._items = items
            self.handle = h
        self._dirty = False

    def __del__(self):
        from . import _lib
        bury(*getattr(self, "graphs", {}).values())
        h = getattr(self, "handle", None)
        if h is not None and h.value:
            _lib.lib().pbte_sweep_batch_destroy(h)

    # -- one chunk of columns of every case's cycle ----------------------------
    def _record(self, j0: int, j1: int) -> None:
        """Columns j0..j1-1 of every case: the batched sweep on the current
        stream, then each case's remaining launches of the column on one of
        ``self.lanes`` side streams (forked from and joined back to the
        current stream: in a captured chunk they are parallel branches, so
        the small latency-bound kernels of different cases overlap)."""
        from . import _lib
        L = _lib.lib()
        main = torch.cuda.current_stream()
        s = main.cuda_stream
        for k in self.cases:
            _lib.check(L.pbte_set_done_flag(k["s"].ctx.handle, k["ar"].state.data_ptr()), "set_done_flag")
        try:
            for j in range(j0, j1):
                _lib.check(L.pbte_sweep_batch_run(self.handle, 1, s), "sweep_batch_run")
                swept = torch.cuda.Event()
                swept.record(main)
                used = set()
                for i, k in enumerate(self.cases):
                    if j >= k["cap"]:
                        continue
                    lane = self.lanes[i % len(self.lanes)]
                    if id(lane) not in used:
                        lane.wait_event(swept)
                        used.add(id(lane))
                    with torch.cuda.stream(lane):
                        k["op32"].after_sweep(lane.cuda_stream, done=k["ar"].state)
                        k["ar"].column_tail(j, lane.cuda_stream)
                for lane in self.lanes:
                    if id(lane) in used:
                        main.wait_stream(lane)
        finally:
            for k in self.cases:
                _lib.check(L.pbte_set_done_flag(k["s"].ctx.handle, None), "set_done_flag")

    def _chunk(self, j0: int, j1: int) -> None:
        if not self.use_graphs:
            self._record(j0, j1)
            return
        g = self.graphs.get((j0, j1))
        if g is None:
            with device_lock:
                empty_graveyard()
                torch.cuda.synchronize(self.device)
                g = torch.cuda.CUDAGraph()
                with torch.cuda.graph(g, stream=self.stream, capture_error_mode="thread_local"):
                    self._record(j0, j1)
            self.graphs[(j0, j1)] = g
        g.replay()

    def _lane(self, i: int):
        return torch.cuda.stream(self.lanes[i % len(self.lanes)])

    def step(self, remove_finished: bool = False) -> list[dict]:
        """One outer step of every unfinished case: its FP64 defect decides
        whether it has converged (or reached tmax); the others run one inner
        cycle in lockstep and update.  Returns the cases that finished in this
        step (with ``remove_finished`` they also leave the batch)."""
        from .krylov import _solve_upper, amplification
        from .mixed import refined

        o = self.opts
        dev = self.device
        for i, k in enumerate(self.cases):
            if k["fresh"]:
                s = k["s"]
                s.reset()
                k["op64"].sweeps = k["op32"].sweeps = 0
                k.update(u=torch.zeros(k["op64"].n, dtype=torch.float64, device=dev), history=[], inner=0,
                         done=False, converged=False, fresh=False, started=time.perf_counter(),
                         kappa=None, dnorm=None)
                with self._lane(i):
                    k["fu"] = k["op64"].apply(k["u"])
        live = [(i, k) for i, k in enumerate(self.cases) if not k["done"]]
        for i, k in live:
            with self._lane(i):
                dn = k["dnorm"] if k["dnorm"] is not None else torch.zeros((), dtype=torch.float64, device=dev)
                k["nrm"] = torch.stack([torch.linalg.vector_norm(k["fu"] - k["u"]),
                                        torch.linalg.vector_norm(k["fu"]), dn])
        torch.cuda.synchronize(dev)
        finished = []
        if live:
            norms = torch.stack([k["nrm"] for _, k in live]).cpu().numpy()
            for (_, k), (rn, fn, dn) in zip(live, norms):
                fn = float(fn) or 1.0
                if k["dnorm"] is not None and k["rn"] > 0:
                    # the last correction solved (I - T) d = r for the last defect
                    amp = float(dn) / k["rn"]
                    k["kappa"] = amp if k["kappa"] is None else max(k["kappa"], amp)
                k["rn"] = float(rn)
                k["history"].append(float(rn) / fn)
                if refined(float(rn), fn, k["kappa"], o):
                    k["done"] = k["converged"] = True
                elif k["op64"].sweeps + k["inner"] >= k["s"].case.iteration.tmax:
                    k["done"] = True
                if k["done"]:
                    k["record"] = self._finish(k)
                    finished.append(k)
        if remove_finished and finished:
            self.cases = [k for k in self.cases if not k["done"]]
            self._dirty = True
        if not any(not k["done"] for k in self.cases):
            return finished
        if self._dirty:
            self._rebuild()
        for i, k in enumerate(self.cases):
            with self._lane(i):
                if k["done"]:
                    k["ar"].state.fill_(9)            # every launch of this case returns at once
                else:
                    k["ar"].begin_cycle(k["fu"] - k["u"], k["rn"], o.inner_rtol * k["rn"])
        torch.cuda.synchronize(dev)
        mmax = max(k["cap"] for k in self.cases)
        for j0 in range(0, mmax, self.CHUNK):
            self._chunk(j0, min(mmax, j0 + self.CHUNK))
            states = torch.stack([k["ar"].state[0] for k in self.cases]).cpu().numpy()
            if all(int(v) != 0 or k["done"] or j0 + self.CHUNK >= k["cap"] for v, k in zip(states, self.cases)):
                break
        for i, k in enumerate(self.cases):
            if k["done"]:
                continue
            kk, _, rmat, gam, _, _ = k["ar"].end_cycle()
            k["inner"] += kk
            with self._lane(i):
                if kk:
                    ar = k["ar"]
                    amp = amplification(rmat)
                    k["kappa"] = amp if k["kappa"] is None else max(k["kappa"], amp)
                    y = torch.from_numpy(_solve_upper(rmat, gam[:kk])).to(device=dev, dtype=ar.Q.dtype)
                    d = (ar.Q[:kk].T @ y).to(torch.float64)
                    k["dnorm"] = torch.linalg.vector_norm(d)
                    k["u"] = k["u"] + d
                else:
                    k["dnorm"] = None
                k["fu"] = k["op64"].apply(k["u"])
        return finished

    def _finish(self, k) -> RunRecord:
        s = k["s"]
        with torch.cuda.stream(self.lanes[0]):
            k["op64"].publish()
        torch.cuda.synchronize(self.device)
        s64 = k["op64"].sweeps
        s.ctx.sweep_count += s64 + k["inner"]
        h = k["history"] or [float("nan")]
        return s._record(s64 + k["inner"], k["converged"], np.array(h), np.full(len(h), s.mom.mass),
                         time.perf_counter() - k["started"], "GSIS" if s.acc is not None else
                         ("KRYLOV" if s.case.scheme.method == "krylov" else "CIS"),
                         extra={"fp64_sweeps": s64, "fp32_sweeps": k["inner"], "inner_precision": "fp32",
                                "outer_steps": len(h), "final_defect": h[-1], "kappa": k["kappa"],
                                "batched": len(self.cases)})

    def run(self) -> list[RunRecord]:
        """Solve every case of the batch from zero; the records in the
        solvers' order."""
        torch.cuda.synchronize(self.device)
        t0 = time.perf_counter()
        for k in self.cases:
            k["fresh"] = True
        for _ in range(self.opts.max_outer + 1):
            self.step()
            if all(k["done"] for k in self.cases):
                break
        for k in self.cases:
            if not k["done"]:
                k["done"] = True
                k["record"] = self._finish(k)
        torch.cuda.synchronize(self.device)
        self.wall_clock = time.perf_counter() - t0
        return [k["record"] for k in self.cases]


def tune_batch_shape(solvers, shapes=((4, 64), (8, 64), (2, 128), (4, 128)), reps: int = 3) -> dict:
    """The autotuner for a batch: times one batched sweep of every case at
    each block shape (CUDA events, after a warm-up launch) and returns
    ``{"choice": (groups, width), "ms": {shape: ms}}``."""
    from . import _lib
    from .krylov import FixedPointOperator, cached

    ops = []
    for s in solvers:
        if s.acc is not None:
            from .gsis import GsisFixedPoint
            ops.append(cached(s, "gsis32h", lambda s=s: GsisFixedPoint(s, "fp32", homogeneous=True)))
        else:
            ops.append(cached(s, "fp32h", lambda s=s: FixedPointOperator(s, "fp32", homogeneous=True,
                                                                             integrals=False)))
    items = (_lib.BatchItem * len(ops))(*[op.batch_item(None) for op in ops])
    L = _lib.lib()
    out = {}
    for g, w in shapes:
        h = ctypes.c_void_p()
        rc = L.pbte_sweep_batch_create(len(ops), items, g, w, ctypes.byref(h))
        if rc != 0:
            continue
        st = torch.cuda.current_stream().cuda_stream
        _lib.check(L.pbte_sweep_batch_run(h, 1, st), "sweep_batch_run")
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record()
        for _ in range(reps):
            _lib.check(L.pbte_sweep_batch_run(h, 1, st), "sweep_batch_run")
        b.record()
        b.synchronize()
        out[f"{g}x{w}"] = a.elapsed_time(b) / reps
        L.pbte_sweep_batch_destroy(h)
    best = min(out, key=out.get)
    g, w = (int(v) for v in best.split("x"))
    return {"choice": (g, w), "ms": {k: round(v, 4) for k, v in out.items()}}


def main(argv=None) -> int:
    """``python -m pbte_gb300.batch --instances N [--seed S] [--runs R]``: the
    first N instances of the batched workload's draw solved as one lockstep
    batch (block shape autotuned); one JSON line with the shape timings and
    the batch's wall clock per run."""
    import argparse
    import json

    from .config import batched_instances

    ap = argparse.ArgumentParser(description=main.__doc__)
    ap.add_argument("--instances", type=int, default=16)
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--runs", type=int, default=2)
    a = ap.parse_args(argv)
    solvers = [Solver(c) for c in batched_instances(a.seed, a.instances)]
    tune = tune_batch_shape(solvers)
    batch = LockstepBatch(solvers, shape=tune["choice"])
    walls = []
    for _ in range(a.runs):
        recs = batch.run()
        walls.append(round(batch.wall_clock, 4))
    print(json.dumps({"instances": a.instances, "seed": a.seed, "shape": list(tune["choice"]), "tune_ms": tune["ms"],
                      "wall_s": walls, "converged": int(sum(r.converged for r in recs))}), flush=True)
    return 0


if __name__ == "__main__":
    raise SystemExit(main())
