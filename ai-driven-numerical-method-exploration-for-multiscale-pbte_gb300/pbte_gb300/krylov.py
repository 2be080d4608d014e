"""GMRES on the outer fixed point, on the device (``pybte/krylov.py:55-363``).

One outer step is the affine map ``u -> F(u) = T u + g`` on the state ``u``
(moments, plus the wall emission when there are adiabatic walls); GMRES
solves ``(I - T) u = g`` with one sweep per product.  The Krylov basis, the
state and the products live on the device.

Each restart cycle runs on the device: per Arnoldi column the product (sweep
+ moments + emission), classical Gram-Schmidt applied twice (the reference's
CGS2, FP64) and the Givens rotation with the stopping tests -- the target
residual, the reference's bounded extension once under ``tol * 1e-2``, and
breakdown -- are launches that honour a device stop state, captured in CUDA
graphs of ten columns.  The host sees a cycle's end only: it reads the
triangular factor and residual estimates, updates the iterate and restarts.
Stopping otherwise follows the reference: GMRES to ``tol *
krylov_tol_factor`` (floored at 1e-14 of ``||g||``), a closing sweep, and
convergence decided on the true transport residual.  ``iterations`` counts
sweeps.
"""
from __future__ import annotations

import ctypes
import time

import numpy as np
import torch

from . import _lib
from .device import bury, device_lock, empty_graveyard, sync

__all__ = ["FixedPointOperator", "gmres", "run_krylov"]

_ENOUGH = 1.0e-2
_FLOOR = 1.0e-14


def uses_graphs(solver) -> bool:
    """Products and Arnoldi columns replay captured CUDA graphs unless the
    solver's ``use_graphs`` is False (then the same launches are issued
    directly: no capture cost, for short-lived solves such as served
    requests)."""
    return getattr(solver, "use_graphs", True)


class FixedPointOperator:
    """``u -> F(u)``: scatter into the sweep's inputs, sweep, moments, wall
    emission, gather (``pybte/krylov.py:64-136``).  The state is
    ``[ts, qxs, qys]``, then the adiabatic-wall emission ``flux_wall`` when
    there are adiabatic walls, then, with periodic faces, the partner
    element's DOFs of every periodic face and ordinate (the sweep reads them
    from ``ctx.pbuf``, so one sweep is a function of the state)."""

    def __init__(self, solver, precision: str = "fp64", homogeneous: bool = False, integrals: bool = True):
        s = solver
        self.integrals = integrals
        self.s = s
        self.nd, self.nt = s.ndof, s.n_tris
        self.k = self.nd * self.nt
        self.nmom = 3 * self.k
        self.wall = bool(s.bcdata.has_nonthermalising)
        self.nwall = s.mesh.n_faces * self.nd if self.wall else 0
        self.per = bool(s.bcdata.has_periodic)
        self.npf = int(np.count_nonzero(s.bcdata.periodic_tri >= 0)) if self.per else 0
        if self.per and precision != "fp64":
            raise NotImplementedError("periodic faces: the FP32 product has no periodic state")
        self.nper = s.ndir * self.npf * self.nd
        self.n = self.nmom + self.nwall + self.nper
        dev = s.device
        f64 = dict(dtype=torch.float64, device=dev)
        self.uin = torch.zeros(self.n, **f64)
        self.uout = torch.zeros_like(self.uin)
        self.precision = precision
        self.homogeneous = homogeneous
        self.vdf = s.vdf if precision == "fp64" else torch.zeros(s.vdf.shape, dtype=torch.float32, device=dev)
        self.temp = torch.zeros(self.nt, **f64)
        self.qx = torch.zeros(self.nt, **f64)
        self.qy = torch.zeros(self.nt, **f64)
        self.sweeps = 0
        self.graph = None
        self.stream = torch.cuda.Stream(device=dev)

    def _views(self, u):
        """``(ts, qxs, qys, flux_wall or None, periodic block or None)``
        views of a state-sized buffer."""
        k, m, w = self.k, self.nmom, self.nwall
        fw = u[m:m + w].view(-1, self.nd) if self.wall else None
        per = u[m + w:].view(self.s.ndir, self.npf, self.nd) if self.per else None
        return (u[:k].view(self.nd, self.nt), u[k:2 * k].view(self.nd, self.nt),
                u[2 * k:3 * k].view(self.nd, self.nt), fw, per)

    @staticmethod
    def _ptr(t):
        return t.data_ptr() if t is not None else None

    def _launch(self, s: int, done=None) -> None:
        """The product's launches on stream ``s``; they honour the context's
        stop flag (``done`` is for products with context-free launches)."""
        L = _lib.lib()
        ctx = self.s.ctx.handle
        p = self._ptr
        ts, qxs, qys, fw, per = self._views(self.uin)
        ots, oqxs, oqys, ofw, oper = self._views(self.uout)
        if self.precision == "fp64":
            pbuf = self.s.ctx.pbuf
            if self.per:
                _lib.check(L.pbte_periodic_scatter(ctx, per.data_ptr(), pbuf.data_ptr(), s), "periodic_scatter")
            _lib.check(L.pbte_sweep(ctx, ts.data_ptr(), qxs.data_ptr(), qys.data_ptr(), self.vdf.data_ptr(),
                                    p(fw), pbuf.data_ptr(), int(self.per), s), "sweep")
            _lib.check(L.pbte_moments(ctx, self.vdf.data_ptr(), ots.data_ptr(), oqxs.data_ptr(), oqys.data_ptr(),
                                      self.temp.data_ptr(), self.qx.data_ptr(), self.qy.data_ptr(), s), "moments")
            if self.wall:
                _lib.check(L.pbte_wall_flux(ctx, self.vdf.data_ptr(), ofw.data_ptr(), s), "wall_flux")
            if self.per:
                _lib.check(L.pbte_periodic_gather(ctx, self.vdf.data_ptr(), oper.data_ptr(), s), "periodic_gather")
        else:
            # one call: sources, FP32 sweep, moments and emission with the
            # z-mirror twins folded (self.vdf is scratch here)
            ints = (self.temp.data_ptr(), self.qx.data_ptr(), self.qy.data_ptr()) if self.integrals \
                else (None, None, None)
            _lib.check(L.pbte_fixed_point_f32(ctx, ts.data_ptr(), qxs.data_ptr(), qys.data_ptr(), p(fw),
                                              0.0 if self.homogeneous else 1.0, self.vdf.data_ptr(),
                                              ots.data_ptr(), oqxs.data_ptr(), oqys.data_ptr(), p(ofw), *ints, s),
                       "fixed_point_f32")

    def batch_item(self, done=None) -> "_lib.BatchItem":
        """This FP32 product's sweep as an item of a batched sweep
        (``pbte_sweep_batch_*``): the inputs are the views of ``uin``, the
        folded distribution is ``vdf``."""
        if self.precision == "fp64" or self.per:
            raise ValueError("only the FP32 product without periodic faces sweeps in a batch")
        ts, qxs, qys, fw, _ = self._views(self.uin)
        return _lib.BatchItem(self.s.ctx.handle.value, ts.data_ptr(), qxs.data_ptr(), qys.data_ptr(),
                              self._ptr(fw), 0.0 if self.homogeneous else 1.0, self.vdf.data_ptr(),
                              None if done is None else done.data_ptr())

    def after_sweep(self, s: int, done=None) -> None:
        """The FP32 product's launches after a batched sweep: moments,
        element integrals and wall emission of the folded distribution."""
        ots, oqxs, oqys, ofw, _ = self._views(self.uout)
        ints = (self.temp.data_ptr(), self.qx.data_ptr(), self.qy.data_ptr()) if self.integrals \
            else (None, None, None)
        _lib.check(_lib.lib().pbte_fold_epilogue_f32(self.s.ctx.handle, self.vdf.data_ptr(), ots.data_ptr(),
                                                     oqxs.data_ptr(), oqys.data_ptr(), self._ptr(ofw), *ints, s),
                   "fold_epilogue_f32")

    def _capture(self):
        with device_lock:
            empty_graveyard()
            torch.cuda.synchronize(self.s.device)
            g = torch.cuda.CUDAGraph()
            with torch.cuda.graph(g, stream=self.stream, capture_error_mode="thread_local"):
                self._launch(torch.cuda.current_stream().cuda_stream)
        self.graph = g

    def __del__(self):
        bury(getattr(self, "graph", None))

    def apply(self, u: torch.Tensor) -> torch.Tensor:
        """F(u), stream-ordered on the current stream."""
        self.uin.copy_(u)
        if uses_graphs(self.s):
            if self.graph is None:
                self._capture()
            self.graph.replay()
        else:
            self._launch(torch.cuda.current_stream().cuda_stream)
        self.sweeps += 1
        return self.uout.clone()

    def state(self) -> torch.Tensor:
        """The state of the solver's current ``vdf`` without sweeping: its
        moments and wall emission, also left in the solver's moments and
        flux buffers (``pybte/krylov.py:128-136``; the restart start)."""
        s = self.s
        L = _lib.lib()
        st = torch.cuda.current_stream().cuda_stream
        u = torch.zeros_like(self.uin)
        ts, qxs, qys, fw, per = self._views(u)
        m = s.mom
        _lib.check(L.pbte_moments(s.ctx.handle, s.vdf.data_ptr(), ts.data_ptr(), qxs.data_ptr(), qys.data_ptr(),
                                  m.temp.data_ptr(), m.qx.data_ptr(), m.qy.data_ptr(), st), "moments")
        m.ts.copy_(ts)
        m.qxs.copy_(qxs)
        m.qys.copy_(qys)
        if self.wall:
            _lib.check(L.pbte_wall_flux(s.ctx.handle, s.vdf.data_ptr(), fw.data_ptr(), st), "wall_flux")
            s.ctx.flux_wall.copy_(fw)
        if self.per:
            _lib.check(L.pbte_periodic_gather(s.ctx.handle, s.vdf.data_ptr(), per.data_ptr(), st), "periodic_gather")
        return u

    def publish(self) -> None:
        """Copy the last product's moments into the solver's state."""
        s = self.s
        ts, qxs, qys, fw, _ = self._views(self.uout)
        s.mom.ts.copy_(ts)
        s.mom.qxs.copy_(qxs)
        s.mom.qys.copy_(qys)
        s.mom.temp.copy_(self.temp)
        s.mom.qx.copy_(self.qx)
        s.mom.qy.copy_(self.qy)
        if self.wall:
            s.ctx.flux_wall.copy_(fw)


class ArnoldiGraphs:
    """One Arnoldi column per CUDA graph replay.

    For ``A v = v - (F(v) - g)`` (``g`` None: ``A v = v - F(v)``) the graph of
    column ``j`` copies ``q_j`` into the operator's input, runs the sweep,
    moments and emission, forms ``w = A q_j`` and both Gram-Schmidt passes
    against ``q_0..q_j``, and leaves ``[h_0..h_j, ||w||]`` in a small device
    buffer: the host reads that buffer once per product (for the Givens
    rotations and the stopping test) instead of driving a dozen launches.
    Graphs are captured on first use of each ``j`` and replayed across
    restarts.

    ``dtype`` is the storage of the basis and of ``w``: float64, or float32
    for the inner solve of the mixed-precision mode, whose operator is an
    FP32 sweep (``pbte_cgs2_f32``).  ``g`` is copied into a buffer the graphs
    read, so the graphs stay valid for a new ``g`` (:meth:`set_g`)."""

    def __init__(self, op: FixedPointOperator, g: torch.Tensor | None, m_cap: int, dtype=torch.float64):
        self.op = op
        n = op.n
        dev = op.s.device
        f64 = dict(dtype=torch.float64, device=dev)
        if m_cap + 1 > _lib.MAX_BASIS:
            raise ValueError(f"device GMRES holds a basis of at most {_lib.MAX_BASIS - 1} vectors")
        self.n = n
        self.m_cap = m_cap
        self.dtype = dtype
        self.Q = torch.zeros((m_cap + 1, n), dtype=dtype, device=dev)
        self.w = torch.zeros(n, dtype=dtype, device=dev)
        self.h = torch.zeros(m_cap + 2, **f64)
        self.scratch = torch.zeros(_lib.cgs2_scratch(m_cap + 1), **f64)   # block partials and ticket
        self.h_host = torch.zeros(m_cap + 2, dtype=torch.float64, pin_memory=True)
        self.g = None if g is None else g.detach().clone()
        self.cycle_graphs = None
        self.stream = torch.cuda.Stream(device=dev)
        #: a left preconditioner M (a callable on device vectors) makes the
        #: products M A q; its torch work cannot skip on the device stop
        #: state, so such a cycle is issued a column at a time
        self.precond = None

    def set_g(self, g: torch.Tensor) -> None:
        self.g.copy_(g)

    def __del__(self):
        bury(*(getattr(self, "cycle_graphs", None) or {}).values())

    #: columns per captured chunk of a cycle (the host checks the stop state
    #: after each chunk)
    CHUNK = 10
    #: a chunk of a cycle with the FP32 product and basis is issued by one
    #: native call (``pbte_gmres_columns_f32``) instead of four calls per
    #: column from Python: the same launches, recorded and issued faster
    native_columns = True

    def _cycle_buffers(self) -> None:
        if getattr(self, "cycle_graphs", None) is not None:
            return
        dev = self.op.s.device
        f64 = dict(dtype=torch.float64, device=dev)
        m = self.m_cap
        self.R = torch.zeros((m, m), **f64)          # row j: column j of the triangular factor
        self.cs = torch.zeros(m, **f64)
        self.sn = torch.zeros(m, **f64)
        self.gam = torch.zeros(m + 1, **f64)
        self.hist = torch.zeros(m, **f64)
        self.tol = torch.zeros(2, **f64)             # [target, enough (< 0: no extension rule)]
        self.state = torch.zeros(4, dtype=torch.int32, device=dev)
        self.state_host = torch.zeros(4, dtype=torch.int32, pin_memory=True)
        self.tol_host = torch.zeros(2, dtype=torch.float64, pin_memory=True)
        self.cycle_graphs = {}

    def _cycle_desc(self):
        """The buffers of a cycle with the FP32 product and FP32 basis, for
        ``pbte_gmres_columns_f32`` (which issues a chunk's launches from
        native code); None for the other forms."""
        op = self.op
        if (op.precision == "fp64" or self.dtype != torch.float32 or op.per
                or not getattr(op, "native_product", True)):
            return None
        p = op._ptr
        ts, qxs, qys, fw, _ = op._views(op.uin)
        ots, oqxs, oqys, ofw, _ = op._views(op.uout)
        ints = (op.temp, op.qx, op.qy) if op.integrals else (None, None, None)
        return _lib.GmresCycleF32(
            ts.data_ptr(), qxs.data_ptr(), qys.data_ptr(), p(fw), 0.0 if op.homogeneous else 1.0,
            op.vdf.data_ptr(), ots.data_ptr(), oqxs.data_ptr(), oqys.data_ptr(), p(ofw), *(p(t) for t in ints),
            self.Q.data_ptr(), self.Q.stride(0), op.uout.data_ptr(), p(self.g), op.uin.data_ptr(),
            self.w.data_ptr(), self.n, self.h.data_ptr(), self.scratch.data_ptr(), self.scratch.numel(),
            self.R.data_ptr(), self.m_cap, self.cs.data_ptr(), self.sn.data_ptr(), self.gam.data_ptr(),
            self.tol.data_ptr(), self.state.data_ptr(), self.hist.data_ptr())

    def _record_cycle(self, j0: int, j1: int, bounded: bool) -> None:
        """Columns j0..j1-1: product, CGS2, rotation and stopping tests, next
        basis vector; all of it skipped on the device once the stop state is
        set (the state is the context's stop flag meanwhile)."""
        L = _lib.lib()
        s = torch.cuda.current_stream().cuda_stream
        ctx, op = self.op.s.ctx.handle, self.op
        if self.native_columns and not bounded and self.precond is None:
            if getattr(self, "_desc", None) is None:
                self._desc = self._cycle_desc()
            if self._desc is not None:
                _lib.check(L.pbte_gmres_columns_f32(ctx, ctypes.byref(self._desc), j0, j1, s), "gmres_columns_f32")
                return
        _lib.check(L.pbte_set_done_flag(ctx, self.state.data_ptr()), "set_done_flag")
        try:
            for j in range(j0, j1):
                op._launch(s, done=self.state)
                self.column_tail(j, s, bounded)
        finally:
            _lib.check(L.pbte_set_done_flag(ctx, None), "set_done_flag")

    def column_tail(self, j: int, s: int, bounded: bool = False) -> None:
        """Column j after its product is in the operator's output: w (with
        the preconditioner, if any), CGS2, the rotation with the stopping
        tests, and the next basis vector; all skipped on the device once the
        stop state is set."""
        L = _lib.lib()
        op, n = self.op, self.n
        g = self.g.data_ptr() if self.g is not None else None
        ldq = self.Q.stride(0)
        if self.precond is not None:
            # w = M (q_j - (F(q_j) - g)), then CGS2 in place
            v = self.Q[j] - (op.uout[:n] - (self.g if self.g is not None else 0.0))
            self.w.copy_(self.precond(v))
            _lib.check(L.pbte_cgs2(self.Q.data_ptr(), ldq, j + 1, self.w.data_ptr(), n, self.h.data_ptr(),
                                   self.scratch.data_ptr(), self.scratch.numel(), s), "cgs2")
            _lib.check(L.pbte_gmres_givens_bounded(j, self.h.data_ptr(), self.R.data_ptr(), self.m_cap,
                                                   self.cs.data_ptr(), self.sn.data_ptr(), self.gam.data_ptr(),
                                                   self.tol.data_ptr(), self.state.data_ptr(),
                                                   self.hist.data_ptr(), s), "gmres_givens_bounded")
        elif self.dtype == torch.float64:
            _lib.check(L.pbte_arnoldi_column_givens(
                self.Q.data_ptr(), ldq, j + 1, op.uout.data_ptr(), g, self.w.data_ptr(), n,
                self.h.data_ptr(), self.scratch.data_ptr(), self.scratch.numel(), self.R.data_ptr(),
                self.m_cap, self.cs.data_ptr(), self.sn.data_ptr(), self.gam.data_ptr(), self.tol.data_ptr(),
                self.state.data_ptr(), self.hist.data_ptr(), int(bounded), s), "arnoldi_column_givens")
        else:
            _lib.check(L.pbte_arnoldi_column_f32(self.Q.data_ptr(), ldq, j + 1, op.uout.data_ptr(), g,
                                                 self.w.data_ptr(), n, self.h.data_ptr(),
                                                 self.scratch.data_ptr(), self.scratch.numel(),
                                                 self.state.data_ptr(), s), "arnoldi_column_f32")
            giv = L.pbte_gmres_givens_bounded if bounded else L.pbte_gmres_givens
            _lib.check(giv(j, self.h.data_ptr(), self.R.data_ptr(), self.m_cap, self.cs.data_ptr(),
                           self.sn.data_ptr(), self.gam.data_ptr(), self.tol.data_ptr(),
                           self.state.data_ptr(), self.hist.data_ptr(), s), "gmres_givens")
        nb = L.pbte_gmres_next_basis_f32 if self.dtype == torch.float32 else L.pbte_gmres_next_basis
        if j + 1 < self.m_cap:
            _lib.check(nb(j, self.w.data_ptr(), self.h.data_ptr(), self.Q.data_ptr(), ldq,
                          op.uin.data_ptr(), n, self.state.data_ptr(), s), "gmres_next_basis")

    def _chunk(self, j0: int, j1: int, bounded: bool):
        key = (j0, j1, bounded)
        if key not in self.cycle_graphs:
            if uses_graphs(self.op.s) and self.precond is None:
                with device_lock:
                    empty_graveyard()
                    torch.cuda.synchronize(self.op.s.device)
                    gr = torch.cuda.CUDAGraph()
                    with torch.cuda.graph(gr, stream=self.stream, capture_error_mode="thread_local"):
                        self._record_cycle(j0, j1, bounded)
                self.cycle_graphs[key] = gr
            else:
                return None
        return self.cycle_graphs[key]

    def cycle(self, r: torch.Tensor, beta: float, m: int, tol_abs: float, rule=None):
        """One restart cycle of at most ``m`` columns from the residual ``r``
        (norm ``beta``), stopping on the device when the residual estimate
        reaches ``tol_abs``, on breakdown, or -- with ``rule = (enough,
        products_before, reached)`` -- by pybte's bounded extension.
        Returns ``(k, stop, R, gam, hist, reached)`` on the host: columns done,
        stop state (0 none, 1 converged, 2 breakdown, 3 halted), the k x k
        triangular factor, the k + 1 residual estimates, the k residual norms
        and the extension's first product under ``enough`` (-1: none)."""
        bounded = rule is not None
        self.begin_cycle(r, beta, tol_abs, rule)
        step = 1 if self.precond is not None else self.CHUNK
        for j0 in range(0, m, step):
            j1 = min(m, j0 + step)
            g = self._chunk(j0, j1, bounded)
            if g is not None:
                g.replay()
            else:
                self._record_cycle(j0, j1, bounded)
            self.state_host.copy_(self.state, non_blocking=True)
            torch.cuda.current_stream().synchronize()
            if int(self.state_host[0]) != 0:
                break
        return self.end_cycle()

    def begin_cycle(self, r: torch.Tensor, beta: float, tol_abs: float, rule=None) -> None:
        """A cycle's start on the current stream: q_0 = r / beta (also the
        operator's input), the residual estimates, the tolerances and the
        stop state (``rule``: see :meth:`cycle`)."""
        self._cycle_buffers()
        n = self.n
        bounded = rule is not None
        torch.div(r, beta, out=self.Q[0])
        self.op.uin[:n].copy_(self.Q[0])
        self.gam.zero_()
        self.gam[0] = beta
        self.tol_host[0] = tol_abs
        self.tol_host[1] = rule[0] if bounded else -1.0
        self.tol.copy_(self.tol_host, non_blocking=True)
        self.state_host.copy_(torch.tensor([0, 0, rule[1] if bounded else 0, rule[2] if bounded else -1],
                                           dtype=torch.int32))
        self.state.copy_(self.state_host, non_blocking=True)

    def end_cycle(self):
        """``(k, stop, R, gam, hist, reached)`` of the finished cycle (reads
        the device state; synchronises)."""
        st = self.state.cpu()
        k = int(st[1])
        R = self.R[:k, :k].cpu().numpy().T.copy()
        gam = self.gam[:k + 1].cpu().numpy()
        hist = self.hist[:k].cpu().numpy()
        self.op.sweeps += k
        return k, int(st[0]), R, gam, hist, int(st[3])

    def capture_all(self) -> None:
        """Capture every chunk of a full device cycle now (capturing
        synchronises the device, which concurrent solves should not meet
        mid-run)."""
        self._cycle_buffers()
        # the FP64 solver's cycles carry the bounded extension, the mixed
        # solver's inner (FP32-product) cycles do not
        bounded = self.op.precision == "fp64"
        for j0 in range(0, self.m_cap, self.CHUNK):
            self._chunk(j0, min(self.m_cap, j0 + self.CHUNK), bounded)


class MomentPreconditioner:
    """Approximate ``(I - T)^-1`` by the GSIS macroscopic system
    (``pybte/krylov.py:369-414``, ``scheme.krylov_precond``): the moment
    blocks of a residual become the source of the HDG local problems, whose
    trace system is solved (with the wall traces of a zero distribution) and
    whose recovered ``T, q_x, q_y`` replace them; the rest of the vector
    passes through.  pybte notes it helps in the diffusive limit and hurts in
    the ballistic one, and leaves it off by default.  The element solves,
    the trace right-hand side and the recovery are the GSIS step's kernels."""

    def __init__(self, solver, acc, sign: float = -1.0):
        self.s = solver
        self.acc = acc
        self.nd, self.nt = solver.ndof, solver.n_tris
        self.k = self.nd * self.nt
        self.sign = sign
        self.calls = 0
        f64 = dict(dtype=torch.float64, device=solver.device)
        self.zero_vdf = torch.zeros_like(solver.vdf)
        self.work = torch.zeros((self.nt, 7 * self.nd), **f64)
        self.src = torch.zeros((self.nt, 7 * self.nd), **f64)
        self.uq = torch.zeros((7 * self.nd, self.nt), **f64)

    def __call__(self, r: torch.Tensor) -> torch.Tensor:
        a, nd, nt, k = self.acc, self.nd, self.nt, self.k
        s = torch.cuda.current_stream().cuda_stream
        # rows 0..2 of each element's local source: T, q_x, q_y of the residual
        self.work[:, :3 * nd].copy_((self.sign * r[:3 * k]).view(3 * nd, nt).T)
        _lib.check(_lib.lib().pbte_gsis_apply_inverse(ctypes.byref(a.ops), self.work.data_ptr(), 0, 3 * nd,
                                                      self.src.data_ptr(), None, s), "gsis_apply_inverse")
        a.rhs(self.src, self.zero_vdf)
        a.trace_solve()
        a.recover(self.src, self.uq)
        out = r.clone()
        out[:3 * k] = self.uq[:3 * nd].reshape(-1)
        self.calls += 1
        return out


def _solve_upper(rmat: np.ndarray, rhs: np.ndarray) -> np.ndarray:
    """``y`` with ``R y = rhs`` for the upper-triangular cycle factor, rows
    from the last up; a zero diagonal gives a zero component (pybte's
    ``_back_substitute``, ``krylov.py:142-147``, the same operation order)."""
    y = np.array(rhs, dtype=float)
    for i in range(y.size - 1, -1, -1):
        t = y[i] - rmat[i, i + 1:] @ y[i + 1:]
        y[i] = t / rmat[i, i] if rmat[i, i] != 0.0 else 0.0
    return y


class Extension:
    """The stopping rule ``run_krylov`` wraps around GMRES
    (``pybte/krylov.py:332-338``): after the first product whose residual is
    under ``enough``, at most ``max(64, reached // 4)`` more products.
    ``count`` is the index of the latest product among the run's products;
    the device applies the same rule inside a cycle
    (``pbte_gmres_givens_bounded``)."""

    def __init__(self, enough: float, count: int):
        self.enough = enough
        self.count = count
        self.reached = -1

    def observe(self, res: float) -> bool:
        """One more product with residual ``res``; True: halt."""
        self.count += 1
        if self.reached < 0 and res <= self.enough:
            self.reached = self.count
        return self.reached >= 0 and self.count - self.reached > max(64, self.reached // 4)


def amplification(R: np.ndarray) -> float:
    """``1 / sigma_min`` of a cycle's ``R`` (the Givens-reduced Arnoldi
    Hessenberg matrix, whose singular values are ``H_k``'s): the norm of
    ``A^-1`` on the Krylov space the cycle explored, which holds the slow
    modes GMRES had to resolve."""
    if R.size == 0:
        return 0.0
    smin = float(np.linalg.svd(R, compute_uv=False)[-1])
    return 1.0 / smin if smin > 0 else float("inf")


def gmres(matvec, b: torch.Tensor, arnoldi: ArnoldiGraphs, x0=None, tol_abs: float = 0.0, maxiter=None,
          rule: Extension | None = None, on_products=None, on_cycle=None):
    """Restarted GMRES for ``A x = b`` (``pybte/krylov.py:150-246``) with its
    restart cycles on the device (:meth:`ArnoldiGraphs.cycle`, basis of at
    most ``arnoldi.m_cap`` vectors).  The host forms each restart's residual
    ``b - A x`` (one product, through ``matvec``; with ``arnoldi.precond`` M
    its ``M (b - A x)``), runs a cycle and adds the cycle's correction
    ``Q_k y`` with ``R y = gam``.  ``rule``: the bounded extension, applied to
    the restart residuals here and to the cycle's columns on the device.
    ``on_products(residuals)``: the residual norms of the products just done,
    in order (a restart's residual, then a cycle's columns).
    ``on_cycle(R)``: each cycle's k x k triangular factor.  Returns ``(x,
    converged, products)``."""
    ar = arnoldi
    x = torch.zeros_like(b) if x0 is None else x0.clone()
    budget = int(b.numel() if maxiter is None else maxiter)
    pre = ar.precond if ar.precond is not None else (lambda v: v)
    done = 0
    converged = False
    while done < budget:
        if bool(torch.any(x != 0).item()):
            r = pre(b - matvec(x))
            done += 1
            beta = float(torch.linalg.vector_norm(r).item())
            if on_products is not None:
                on_products([beta])
            if rule is not None and rule.observe(beta):
                break
        else:
            r = pre(b.clone())
            beta = float(torch.linalg.vector_norm(r).item())
        if beta <= tol_abs:
            converged = True
            break
        m = min(ar.m_cap, budget - done)
        if m <= 0:
            break
        k, stop, rmat, gam, hist, reached = ar.cycle(
            r, beta, m, tol_abs, None if rule is None else (rule.enough, rule.count, rule.reached))
        done += k
        if rule is not None:
            rule.count += k
            rule.reached = reached
        if on_products is not None and k:
            on_products(list(hist))
        if k:
            if on_cycle is not None:
                on_cycle(rmat)
            y = torch.from_numpy(_solve_upper(rmat, gam[:k])).to(device=b.device, dtype=ar.Q.dtype)
            x += (ar.Q[:k].T @ y).to(x.dtype)
        if stop == 1:
            converged = True
            break
        if stop == 3:
            break
    return x, converged, done


def cached(solver, key, make):
    """Operators and Arnoldi graphs kept on the solver across runs: their
    CUDA graphs hold the context's and the solver's buffers, so an entry is
    rebuilt when the solver has a new context or distribution buffer."""
    cache = solver.__dict__.setdefault("_krylov_cache", {})
    hit = cache.get(key)
    if hit is None or hit[0] is not solver.ctx or hit[1] != solver.vdf.data_ptr():
        hit = (solver.ctx, solver.vdf.data_ptr(), make())
        cache[key] = hit
    return hit[2]


def basis_cap(case, n: int) -> int:
    """pybte's Krylov dimension (``krylov.py:249-251``: ``krylov_restart``,
    else what ``krylov_max_bytes`` holds, at least 32 and at most ``tmax``),
    held to the device basis limit (``PBTE_MAX_BASIS - 1`` vectors)."""
    return min(requested_basis(case, n), _lib.MAX_BASIS - 1)


def requested_basis(case, n: int) -> int:
    if case.scheme.krylov_restart is not None:
        return int(case.scheme.krylov_restart)
    per = max(1.0, 8.0 * float(n))
    return int(max(32, min(int(case.iteration.tmax), int(case.scheme.krylov_max_bytes / per))))


def run_krylov(solver, callback=None, progress_every: int = 0):
    """``pybte/krylov.py:257-363`` on the device.  ``callback(step,
    residual, solver)`` and progress lines follow every residual, in order;
    the products of a restart cycle are reported when the cycle ends.  A
    restarted solver starts GMRES from its loaded state."""
    c = solver.case
    tol, tmax = c.iteration.tol, c.iteration.tmax
    want_true = c.iteration.true_residual
    op = cached(solver, "fp64", lambda: FixedPointOperator(solver))
    op.sweeps = 0
    residuals, true_res = [], []

    def report(values):
        for v in values:
            residuals.append(v)
            if want_true:
                true_res.append(np.nan)
            step = len(residuals)
            if progress_every and step % progress_every == 0:
                print(f"  step {step:8d}  residual {v:.6e}", flush=True)
            if callback is not None:
                callback(step, v, solver)

    sync(solver.device)
    t0 = time.perf_counter()
    restarted = bool(solver.restart_info.get("enabled")) if hasattr(solver, "restart_info") else False
    x = op.state() if restarted else torch.zeros(op.n, dtype=torch.float64, device=solver.device)
    g = op.apply(torch.zeros(op.n, dtype=torch.float64, device=solver.device))
    gnorm = float(torch.linalg.vector_norm(g).item())
    scale = gnorm or 1.0
    report([1.0])

    def matvec(v):
        return v - (op.apply(v) - g)

    enough = max(tol * _ENOUGH, _FLOOR) * scale
    target = max(tol * c.scheme.krylov_tol_factor, _FLOOR) * scale
    cap = basis_cap(c, op.n)
    ar = cached(solver, ("arnoldi64", cap), lambda: ArnoldiGraphs(op, g, cap))
    ar.set_g(g)
    precond = None
    if c.scheme.krylov_precond and getattr(solver, "acc", None) is not None:
        precond = MomentPreconditioner(solver, solver.acc)
    ar.precond = precond
    converged = False
    final = float("nan")
    for _ in range(c.scheme.krylov_max_rounds):
        budget = tmax - len(residuals) - 1
        if budget <= 0:
            break
        x, _, _ = gmres(matvec, g, ar, x0=x, tol_abs=target, maxiter=budget,
                        rule=Extension(enough, len(residuals)), on_products=lambda v: report([e / scale for e in v]))
        op.apply(x)                                       # closing sweep
        op.publish()
        final = solver.ctx.true_residual(solver.mom, solver.vdf)
        report([final])
        if want_true:
            true_res[-1] = final
        converged = bool(final < tol) if np.isfinite(final) else gnorm == 0.0
        if converged or len(residuals) >= tmax:
            break
        target = max(target * 1.0e-3, _FLOOR * scale)
    ar.precond = None
    sync(solver.device)
    wall = time.perf_counter() - t0
    solver.ctx.sweep_count += op.sweeps
    masses = [solver.mom.mass] * len(residuals)
    return solver._record(len(residuals), converged, residuals, masses, wall, "KRYLOV",
                          extra={"krylov_size": op.n, "krylov_periodic_state": op.nper, "krylov_basis_cap": cap,
                                 "krylov_basis_requested": requested_basis(c, op.n),
                                 "krylov_precond": precond is not None, "transport_residual": final},
                          true_res=true_res if want_true else None)
