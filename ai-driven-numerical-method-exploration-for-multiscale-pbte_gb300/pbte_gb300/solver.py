"""Outer iterations on the GPU behind pybte's ``Solver`` interface.

``Solver(case).run()`` returns a :class:`RunRecord`, as pybte's does
(``pybte/driver.py:43-254``):

* ``scheme.method = "source"``, ``accflag = 0`` -- CIS (``driver.py:170-215``).
  One outer iteration is [wall emission] -> sweep -> moments -> step residual
  -> stopping rule, all on the device; a block of iterations is captured once
  as a CUDA graph and replayed, with a device-side stop flag so the run ends
  on exactly the iteration where the residual first drops under ``tol``.
* ``accflag = 1`` -- GSIS (:mod:`pbte_gb300.gsis`).
* ``scheme.method = "krylov"`` -- GMRES on the outer fixed point
  (``pybte/krylov.py:257-363``), basis on the device, one sweep per product.

``performance.precision = "mixed"`` runs the same scheme with FP32 sweeps
inside an FP64 defect-correction loop (:mod:`pbte_gb300.mixed`).
"""
from __future__ import annotations

import ctypes
import time
from dataclasses import dataclass, field

import numpy as np
import torch

from . import _lib
from .config import Case
from .device import bury, device_lock, empty_graveyard, sync
from .discretisation import Discretisation
from .sweep import Moments, SweepContext

__all__ = ["Solver", "RunRecord"]


@dataclass
class RunRecord:
    """The fields of pybte's ``RunRecord`` (``pybte/io_output.py:30-164``)
    that describe a solve; arrays are host numpy."""
    iterations: int
    converged: bool
    residual_history: np.ndarray
    mass_history: np.ndarray
    temp: np.ndarray
    qx: np.ndarray
    qy: np.ndarray
    temp_dofs: np.ndarray
    qx_dofs: np.ndarray
    qy_dofs: np.ndarray
    sweep_count: int
    wall_clock: float
    setup_wall_clock: float
    scheme: str
    tol: float
    tau_r: float
    tau_n: float
    deg: int
    npole: int
    nazim: int
    n_tris: int
    precision: str = "fp64"
    residual_true: np.ndarray | None = None
    diagnostics: dict = field(default_factory=dict)

    @property
    def mass(self) -> float:
        return float(np.sum(self.temp))


class Solver:
    """Set up a case on the GPU and run it to convergence."""

    def __init__(self, case: Case, device: str = "cuda", graph_block: int = 32,
                 discretisation: Discretisation | None = None):
        t0 = time.perf_counter()
        self.case = case
        self.device = torch.device(device)
        self.disc = discretisation if discretisation is not None else Discretisation.build(case)
        self.mesh, self.integrals, self.vel = self.disc.mesh, self.disc.integrals, self.disc.vel
        self.bcdata = self.disc.bcdata
        self.ndir, self.n_tris, self.ndof = self.disc.ndir, self.disc.n_tris, self.disc.ndof
        self.precision = case.performance.precision
        self.ctx = SweepContext(self.disc, device=device)
        f64 = dict(dtype=torch.float64, device=self.device)
        self.vdf = torch.zeros((self.ndir, self.n_tris, self.ndof), **f64)
        self.mom = Moments.zeros(self.ndof, self.n_tris, device=self.device)
        self.t_old = torch.zeros(self.n_tris, **f64)
        self._res = torch.zeros(2, **f64)
        self.graph_block = int(graph_block)
        self.acc = None
        if case.scheme.accflag == 1:
            from .gsis import GSIS
            self.acc = GSIS(self)
        sync(self.device)
        self.setup_seconds = time.perf_counter() - t0

    def release(self) -> None:
        """Free the solver's device state now -- Krylov operators and their
        graphs, the acceleration, the context -- under the device lock, so
        nothing is destroyed while another thread captures a graph.  The
        solver is unusable afterwards."""
        with device_lock:
            self.__dict__.pop("_krylov_cache", None)
            self.acc = None
            ctx = self.__dict__.pop("ctx", None)
            del ctx
            empty_graveyard()

    def reset(self) -> None:
        """Back to the zero initial state of a fresh solve (on the current
        stream)."""
        self.vdf.zero_()
        for k in ("ts", "qxs", "qys", "temp", "qx", "qy"):
            getattr(self.mom, k).zero_()
        self.t_old.zero_()
        self.ctx.flux_wall.zero_()

    # -- one outer iteration (pybte/driver.py:149-161) -----------------------
    def step(self, stream=None) -> None:
        if self.bcdata.has_nonthermalising:
            self.ctx.wall_flux(self.vdf, stream=stream)
        self.ctx.sweep(self.mom, self.vdf, stream=stream)
        if self.acc is None:
            self.ctx.moments(self.vdf, self.mom, stream=stream)
        else:
            self.acc.apply(stream=stream)

    def run(self, callback=None, progress_every: int = 0) -> RunRecord:
        c = self.case
        if self.precision == "mixed":
            from .mixed import run_mixed
            return run_mixed(self)
        if c.scheme.method == "krylov":
            from .krylov import run_krylov
            return run_krylov(self)
        if self.acc is not None:
            return self._run_stepwise("GSIS")
        return self._run_source()

    # -- CIS, graph-captured ------------------------------------------------
    def _iteration(self, s: int, tol: float, tmax: int, done, count, hist, cap) -> None:
        L = _lib.lib()
        ctx = self.ctx.handle
        if self.bcdata.has_nonthermalising:
            _lib.check(L.pbte_wall_flux(ctx, self.vdf.data_ptr(), self.ctx.flux_wall.data_ptr(), s), "wall_flux")
        m = self.mom
        _lib.check(L.pbte_sweep(ctx, m.ts.data_ptr(), m.qxs.data_ptr(), m.qys.data_ptr(), self.vdf.data_ptr(),
                                self.ctx.flux_wall.data_ptr(), self.ctx.pbuf.data_ptr(), 0, s), "sweep")
        _lib.check(L.pbte_moments(ctx, self.vdf.data_ptr(), m.ts.data_ptr(), m.qxs.data_ptr(), m.qys.data_ptr(),
                                  m.temp.data_ptr(), m.qx.data_ptr(), m.qy.data_ptr(), s), "moments")
        _lib.check(L.pbte_residual_iterate(ctx, m.temp.data_ptr(), self.t_old.data_ptr(),
                                           self._res.data_ptr(), s), "residual")
        _lib.check(L.pbte_residual_check(ctx, self._res.data_ptr(), float(tol), int(tmax), done.data_ptr(),
                                         count.data_ptr(), hist.data_ptr(), int(cap), s), "check")

    def _run_source(self) -> RunRecord:
        c = self.case
        tol, tmax = c.iteration.tol, c.iteration.tmax
        dev = self.device
        done = torch.zeros(1, dtype=torch.int32, device=dev)
        count = torch.zeros(1, dtype=torch.int64, device=dev)
        cap = min(int(tmax), 1 << 22)
        hist = torch.zeros(2 * cap, dtype=torch.float64, device=dev)
        L = _lib.lib()
        _lib.check(L.pbte_set_done_flag(self.ctx.handle, done.data_ptr()), "set_done_flag")
        K = max(1, min(self.graph_block, int(tmax)))
        stream = torch.cuda.Stream(device=dev)
        sync(dev)
        t0 = time.perf_counter()
        g = None
        try:
            g = torch.cuda.CUDAGraph()
            with device_lock:
                empty_graveyard()
                with torch.cuda.graph(g, stream=stream, capture_error_mode="thread_local"):
                    s = torch.cuda.current_stream().cuda_stream
                    for _ in range(K):
                        self._iteration(s, tol, tmax, done, count, hist, cap)
            while True:
                g.replay()
                if int(done.item()) != 0:
                    break
        finally:
            _lib.check(L.pbte_set_done_flag(self.ctx.handle, None), "set_done_flag")
            bury(g)
        sync(dev)
        wall = time.perf_counter() - t0
        n = int(count.item())
        flag = int(done.item())
        self.ctx.sweep_count += n
        h = hist[:2 * min(n, cap)].cpu().numpy().reshape(-1, 2)
        return self._record(n, flag == 1, h[:, 0], h[:, 1], wall, "CIS")

    # -- host-driven loop (GSIS and debugging) -------------------------------
    def _run_stepwise(self, scheme: str) -> RunRecord:
        c = self.case
        tol, tmax = c.iteration.tol, c.iteration.tmax
        L = _lib.lib()
        residuals, masses = [], []
        sync(self.device)
        t0 = time.perf_counter()
        step, converged = 0, False
        s = torch.cuda.current_stream().cuda_stream
        while True:
            step += 1
            self.step()
            _lib.check(L.pbte_residual_iterate(self.ctx.handle, self.mom.temp.data_ptr(), self.t_old.data_ptr(),
                                               self._res.data_ptr(), s), "residual")
            r = self._res.cpu().numpy()
            residuals.append(float(r[0]))
            masses.append(float(r[1]))
            if r[0] < tol:
                converged = True
                break
            if step >= tmax:
                break
        sync(self.device)
        wall = time.perf_counter() - t0
        return self._record(step, converged, np.array(residuals), np.array(masses), wall, scheme)

    def _record(self, iterations, converged, residuals, masses, wall, scheme, extra=None) -> RunRecord:
        c = self.case
        h = self.mom.host()
        rec = RunRecord(iterations=int(iterations), converged=bool(converged),
                        residual_history=np.asarray(residuals), mass_history=np.asarray(masses),
                        temp=h["temp"], qx=h["qx"], qy=h["qy"], temp_dofs=h["ts"], qx_dofs=h["qxs"],
                        qy_dofs=h["qys"], sweep_count=self.ctx.sweep_count, wall_clock=wall,
                        setup_wall_clock=self.setup_seconds, scheme=scheme, tol=c.iteration.tol,
                        tau_r=c.flow.tau_r, tau_n=c.flow.tau_n, deg=c.dg.deg,
                        npole=c.velmesh.npole, nazim=c.velmesh.nazim, n_tris=self.n_tris,
                        precision=self.precision,
                        diagnostics={"sweep_mode": self.ctx.mode, "n_classes": self.ctx.n_classes,
                                     "n_levels_max": self.ctx.n_levels_max,
                                     "device_bytes": self.ctx.device_bytes,
                                     "boundary_types": [b.type for b in c.boundaries]})
        if extra:
            rec.diagnostics.update(extra)
        return rec

    def true_residual(self) -> float:
        return self.ctx.true_residual(self.mom, self.vdf)
