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

import threading
import time

import torch

from .krylov import ArnoldiGraphs
from .solver import RunRecord, Solver

__all__ = ["BatchSolver"]


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
