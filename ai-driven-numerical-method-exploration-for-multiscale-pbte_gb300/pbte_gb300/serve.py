"""Serving: continuous batching of solve requests on one GPU.

Requests (cases) arrive over time.  The admission thread takes them in
arrival order and admits the oldest waiting request as soon as a solve slot
is free and its device memory (estimated from the discretisation before
anything is allocated) fits in what the running solves leave of the HBM
budget.  Every admitted solve runs on its own CUDA stream and host thread
(as in :mod:`pbte_gb300.batch`), with its operators, iterates and Krylov
basis resident on the device until it completes; then its memory returns to
the budget and the next request is admitted.  Solves that are in flight at
the same time overlap on the device; each result is the one the case gives
alone (no buffer is shared between solves, and every kernel is
deterministic).

With ``mode="lockstep"`` (mixed-precision requests) the admitted solves
are batched continuously into one :class:`pbte_gb300.batch.LockstepBatch`:
an engine thread advances every admitted solve by one outer step at a time,
all their inner FP32 products swept in one launch per DG order; a request
whose set-up (done on its own host thread) has finished joins the batch at
the next step, and a finished one leaves it and returns its memory to the
budget.

Latency of a request = completion time - arrival time (queueing, setup on
the host and the device, and the solve).
"""
from __future__ import annotations

import threading
import time
from dataclasses import dataclass, field

import numpy as np
import torch

from .config import Case, square_case
from .discretisation import Discretisation
from .solver import RunRecord, Solver

__all__ = ["Server", "Ticket", "estimate_device_bytes", "draw_cases"]


def estimate_device_bytes(disc: Discretisation, case: Case) -> int:
    """Upper estimate of the device memory one solve of ``case`` holds:
    distributions, stored factors, sweep records, moment partials, Krylov
    basis and vectors, with a 25 % margin."""
    nd, nt, ndir, nf = disc.ndof, disc.n_tris, disc.ndir, disc.mesh.n_faces
    b = 8.0 * ndir * nt * nd                                   # FP64 distribution
    mixed = case.performance.precision == "mixed"
    if mixed:
        b += 4.0 * ndir * nt * nd                              # FP32 distribution
    if case.performance.precompute_inverse and case.performance.sweep_mode != "onthefly":
        b += (ndir / 2 + 1) * nt * (nd * nd * 8 + nd)          # stored factors, once per velocity pair
    b += 16 * nt * (17 * 12 + 12 * 4)                          # field-major sweep records (<= 16 classes)
    b += ((ndir + 31) // 32) * 3 * nd * nt * 8                 # moment partials
    n = 3 * nd * nt + nf * nd                                  # Krylov state
    cap = case.scheme.krylov_restart or 32
    if case.scheme.method == "krylov":
        b += (cap + 2) * n * (4 if mixed else 8) + 12 * n * 8
    b += 64 * nt * nd * 8 + (64 << 20)                         # moments, scratch, graphs
    return int(1.25 * b)


@dataclass
class Ticket:
    """One request: its case, times (seconds, server clock) and result."""
    case: Case
    arrival: float
    index: int
    admitted: float | None = None
    done: float | None = None
    record: RunRecord | None = None
    error: BaseException | None = None
    bytes: int = 0
    _event: threading.Event = field(default_factory=threading.Event, repr=False)

    def result(self, timeout: float | None = None) -> RunRecord:
        if not self._event.wait(timeout):
            raise TimeoutError("request not finished")
        if self.error is not None:
            raise self.error
        return self.record  # type: ignore[return-value]

    @property
    def latency(self) -> float:
        return (self.done - self.arrival) if self.done is not None else float("nan")


class Server:
    """Admit solve requests by slot and HBM budget; run the admitted ones
    concurrently.  ``submit`` is thread-safe; ``close`` waits for the queue
    to drain."""

    def __init__(self, device: str = "cuda", hbm_budget: float = 150e9, slots: int = 4,
                 ring_shape: tuple[int, int] | None = (4, 64), runner=None, estimator=None,
                 use_graphs: bool = False, mode: str = "streams", batch_shape: tuple[int, int] = (2, 128)):
        if mode not in ("streams", "lockstep"):
            raise ValueError("mode is 'streams' or 'lockstep'")
        self.mode = mode
        self.batch_shape = batch_shape
        self.device = torch.device(device)
        self.budget = int(hbm_budget)
        self.slots = int(slots)
        self.ring_shape = ring_shape
        # a served solve lives for one run: capturing a graph per Arnoldi
        # column costs more than it saves, and each capture holds the
        # device lock that the other requests' captures wait on
        self.use_graphs = use_graphs
        # runner(case, disc) -> RunRecord and estimator(disc, case) -> bytes;
        # replaceable so the admission logic can be exercised without a GPU
        self.runner = runner or self._run_on_device
        self.estimator = estimator or estimate_device_bytes
        self._lock = threading.Condition()
        self._pending: list[Ticket] = []
        self._running = 0
        self._used = 0
        self._closed = False
        self._count = 0
        self.tickets: list[Ticket] = []
        self.t0 = time.perf_counter()
        self.peak_used = 0
        self.peak_running = 0
        self._ready: list = []          # (ticket, solver) set up and waiting to join the batch
        self._admitter = threading.Thread(target=self._admit_loop, daemon=True)
        self._admitter.start()
        self._engine = None
        if mode == "lockstep":
            self._engine = threading.Thread(target=self._engine_loop, daemon=True)
            self._engine.start()

    def now(self) -> float:
        return time.perf_counter() - self.t0

    def submit(self, case: Case) -> Ticket:
        with self._lock:
            if self._closed:
                raise RuntimeError("server closed")
            t = Ticket(case=case, arrival=self.now(), index=self._count)
            self._count += 1
            self._pending.append(t)
            self.tickets.append(t)
            self._lock.notify_all()
        return t

    def close(self) -> None:
        with self._lock:
            self._closed = True
            self._lock.notify_all()
        self._admitter.join()
        with self._lock:
            while self._running:
                self._lock.wait()
            self._lock.notify_all()
        if self._engine is not None:
            self._engine.join()

    # -- admission ---------------------------------------------------------
    def _admit_loop(self) -> None:
        while True:
            with self._lock:
                while not self._pending and not self._closed:
                    self._lock.wait()
                if not self._pending and self._closed:
                    return
                t = self._pending[0]
            # the discretisation is built on the host outside the lock
            try:
                disc = Discretisation.build(t.case)
                need = int(self.estimator(disc, t.case))
            except BaseException as e:   # reported on the ticket
                with self._lock:
                    self._pending.pop(0)
                t.error, t.done = e, self.now()
                t._event.set()
                continue
            with self._lock:
                if need > self.budget:
                    self._pending.pop(0)
                    t.error = MemoryError(f"request needs ~{need / 1e9:.1f} GB, over the {self.budget / 1e9:.1f} GB budget")
                    t.done = self.now()
                    t._event.set()
                    continue
                while self._running >= self.slots or self._used + need > self.budget:
                    self._lock.wait()
                self._pending.pop(0)
                self._running += 1
                self._used += need
                self.peak_used = max(self.peak_used, self._used)
                self.peak_running = max(self.peak_running, self._running)
                t.bytes, t.admitted = need, self.now()
            target = self._setup if self.mode == "lockstep" else self._solve
            threading.Thread(target=target, args=(t, disc), daemon=True).start()

    def _run_on_device(self, case: Case, disc: Discretisation) -> RunRecord:
        stream = torch.cuda.Stream(device=self.device)
        with torch.cuda.stream(stream):
            s = Solver(case, device=str(self.device), discretisation=disc)
            s.use_graphs = self.use_graphs
            if self.ring_shape is not None:
                s.ctx.set_groups(*self.ring_shape)
            try:
                rec = s.run()
                stream.synchronize()
            finally:
                s.release()
        return rec

    # -- continuous batching ----------------------------------------------------
    def _setup(self, t: Ticket, disc: Discretisation) -> None:
        """Host and device set-up of an admitted request on its own thread;
        the engine adds the solver to the batch at its next step."""
        try:
            s = Solver(t.case, device=str(self.device), discretisation=disc)
            if s.precision != "mixed":
                raise ValueError("lockstep serving batches mixed-precision solves")
        except BaseException as e:   # reported on the ticket
            self._complete(t, error=e)
            return
        with self._lock:
            self._ready.append((t, s))
            self._lock.notify_all()

    def _complete(self, t: Ticket, record=None, error=None) -> None:
        t.record, t.error = record, error
        t.done = self.now()
        with self._lock:
            self._running -= 1
            self._used -= t.bytes
            self._lock.notify_all()
        t._event.set()

    def _engine_loop(self) -> None:
        from .batch import LockstepBatch

        batch = LockstepBatch(shape=self.batch_shape, use_graphs=False, device=self.device)
        owner = {}
        while True:
            with self._lock:
                while not self._ready and not batch.cases and not (self._closed and self._running == 0):
                    self._lock.wait()
                if not self._ready and not batch.cases and self._closed and self._running == 0:
                    return
                joining, self._ready = self._ready, []
            for t, s in joining:
                k = batch.add(s)
                owner[id(k)] = t
            try:
                finished = batch.step(remove_finished=True)
            except BaseException as e:   # every solve of the failed step reports it
                for k in list(batch.cases):
                    self._complete(owner.pop(id(k)), error=e)
                    k["s"].release()
                batch = LockstepBatch(shape=self.batch_shape, use_graphs=False, device=self.device)
                continue
            for k in finished:
                t = owner.pop(id(k))
                k["s"].release()
                self._complete(t, record=k["record"])

    def _solve(self, t: Ticket, disc: Discretisation) -> None:
        try:
            t.record = self.runner(t.case, disc)
        except BaseException as e:   # reported on the ticket
            t.error = e
        t.done = self.now()
        with self._lock:
            self._running -= 1
            self._used -= t.bytes
            self._lock.notify_all()
        t._event.set()

    # -- reports -------------------------------------------------------------
    def stats(self) -> dict:
        done = [t for t in self.tickets if t.done is not None and t.error is None]
        if not done:
            return {"completed": 0}
        lat = np.array([t.latency for t in done]) * 1e3
        span = max(t.done for t in done) - min(t.arrival for t in done)
        return {"completed": len(done), "failed": sum(t.error is not None for t in self.tickets),
                "p50_ms": float(np.percentile(lat, 50)), "p99_ms": float(np.percentile(lat, 99)),
                "solves_per_s": len(done) / span if span > 0 else float("nan"),
                "peak_concurrent": self.peak_running, "peak_budget_gb": self.peak_used / 1e9}


_NDIR = {64: (4, 16), 128: (8, 16), 256: (8, 32), 512: (8, 64)}


def draw_cases(n: int, seed: int, grids=(16, 32, 64, 128), degs=(1, 2, 3), ndirs=(64, 128, 256, 512),
               log10_tau=(-3.0, 1.0), precision: str = "mixed") -> list[Case]:
    """Uneven square-cavity instances: grid side, DG order, ordinate count
    and log10 Kn_R uniform over the given sets/range (Kn_N = 0.1 Kn_R), wall
    temperature deviation uniform in [0.1, 1] (west +dT, east -dT);
    GMRES(30), tol 1e-8."""
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(n):
        g = int(rng.choice(grids))
        deg = int(rng.choice(degs))
        nd = int(rng.choice(ndirs))
        kn = float(10.0 ** rng.uniform(*log10_tau))
        dt = float(rng.uniform(0.1, 1.0))
        npole, nazim = _NDIR[nd]
        out.append(square_case(g, deg, npole, nazim, tau_r=kn, tau_n=0.1 * kn, method="krylov",
                               precision=precision, krylov_restart=30, tol=1e-8, tmax=20000,
                               t_west=dt, t_east=-dt))
    return out


def main(argv=None) -> int:
    """Open-loop serving run: ``--requests`` instances drawn with ``--seed``,
    Poisson arrivals at ``--rate`` per second; prints one JSON line with the
    latency percentiles and throughput, and with ``--serial-fp64`` the same
    requests solved one after another in FP64 for comparison."""
    import argparse
    import json

    ap = argparse.ArgumentParser(description=main.__doc__)
    ap.add_argument("--requests", type=int, default=24)
    ap.add_argument("--rate", type=float, default=20.0)
    ap.add_argument("--seed", type=int, default=1)
    ap.add_argument("--slots", type=int, default=4)
    ap.add_argument("--budget-gb", type=float, default=150.0)
    ap.add_argument("--grids", default="16,32,64")
    ap.add_argument("--degs", default="1,2")
    ap.add_argument("--ndirs", default="64,128,256")
    ap.add_argument("--log10-tau", default="-1,1")
    ap.add_argument("--serial-fp64", action="store_true")
    ap.add_argument("--mode", default="streams", choices=["streams", "lockstep"])
    ap.add_argument("--batched-draw", action="store_true",
                    help="draw the requests as the batched workload does (GSIS; every grid, order, "
                         "ordinate count and Kn_R in [1e-3, 10])")
    a = ap.parse_args(argv)
    ints = lambda s: tuple(int(x) for x in s.split(","))
    lo, hi = (float(x) for x in a.log10_tau.split(","))
    if a.batched_draw:
        from .config import batched_instances
        cases = batched_instances(a.seed, a.requests)
    else:
        cases = draw_cases(a.requests, a.seed, ints(a.grids), ints(a.degs), ints(a.ndirs), (lo, hi))
    gaps = np.random.default_rng(a.seed + 1000).exponential(1.0 / a.rate, size=len(cases))
    srv = Server(hbm_budget=a.budget_gb * 1e9, slots=a.slots, mode=a.mode)
    for c, gap in zip(cases, gaps):
        time.sleep(float(gap))
        srv.submit(c)
    srv.close()
    out = {"requests": a.requests, "rate_per_s": a.rate, "seed": a.seed, "slots": a.slots, "mode": a.mode,
           **srv.stats()}
    if a.serial_fp64:
        t0 = time.perf_counter()
        lat = []
        if a.batched_draw:
            from .config import batched_instances
            cases64 = batched_instances(a.seed, a.requests, precision="fp64")
        else:
            cases64 = draw_cases(a.requests, a.seed, ints(a.grids), ints(a.degs), ints(a.ndirs), (lo, hi),
                                 precision="fp64")
        for c in cases64:
            t1 = time.perf_counter()
            s = Solver(c)
            s.use_graphs = srv.use_graphs
            s.run()
            s.release()
            lat.append(time.perf_counter() - t1)
        span = time.perf_counter() - t0
        out["serial_fp64"] = {"solves_per_s": len(lat) / span, "p50_ms": float(np.percentile(lat, 50) * 1e3),
                              "p99_ms": float(np.percentile(lat, 99) * 1e3)}
    print(json.dumps(out), flush=True)
    return 0


if __name__ == "__main__":
    raise SystemExit(main())
