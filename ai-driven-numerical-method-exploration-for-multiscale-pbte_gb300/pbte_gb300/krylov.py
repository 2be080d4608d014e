"""GMRES on the outer fixed point, on the device (``pybte/krylov.py:55-363``).

One outer step is the affine map ``u -> F(u) = T u + g`` on the state ``u``
(moments, plus the wall emission when there are adiabatic walls); GMRES
solves ``(I - T) u = g`` with one sweep per product.  The Krylov basis, the
state and the products live on the device; the map ``F`` (sweep + moments +
emission) is captured once as a CUDA graph on fixed input/output buffers.
The Hessenberg column (``j + 2`` numbers) comes to the host each step for the
Givens rotations, as in the reference.

Orthogonalisation is classical Gram-Schmidt applied twice (the reference's
CGS2), in FP64.  Stopping follows the reference: GMRES to
``tol * krylov_tol_factor`` (floored at 1e-14 of ``||g||``), a bounded
extension once under ``tol * 1e-2``, a closing sweep, and convergence
decided on the true transport residual.  ``iterations`` counts sweeps.
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

    def _launch(self, s: int) -> None:
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
        if m_cap + 1 > 64:
            raise ValueError("graph-captured Arnoldi supports a basis of at most 63 vectors")
        self.n = n
        self.m_cap = m_cap
        self.dtype = dtype
        self.Q = torch.zeros((m_cap + 1, n), dtype=dtype, device=dev)
        self.w = torch.zeros(n, dtype=dtype, device=dev)
        self.h = torch.zeros(m_cap + 2, **f64)
        self.scratch = torch.zeros(_lib.CGS2_SCRATCH, **f64)   # block partials and ticket
        self.h_host = torch.zeros(m_cap + 2, dtype=torch.float64, pin_memory=True)
        self.g = None if g is None else g.detach().clone()
        self.graphs = {}
        self.cycle_graphs = None
        self.stream = torch.cuda.Stream(device=dev)
        self.on_product = None   # called after every product (sweep bookkeeping)
        #: whole restart cycles on the device when no per-column host
        #: callback is needed (the mixed path's inner solve)
        self.device_cycles = True

    def set_g(self, g: torch.Tensor) -> None:
        self.g.copy_(g)

    def _record(self, j: int, done=None, fill_input: bool = True) -> None:
        op = self.op
        n = self.n
        Qj = self.Q[:j + 1]
        if fill_input:
            op.uin[:n].copy_(self.Q[j])
        op._launch(torch.cuda.current_stream().cuda_stream)
        L = _lib.lib()
        fn = L.pbte_arnoldi_column_f32 if self.dtype == torch.float32 else L.pbte_arnoldi_column
        g = self.g.data_ptr() if self.g is not None else None
        _lib.check(fn(Qj.data_ptr(), self.Q.stride(0), j + 1, op.uout.data_ptr(), g, self.w.data_ptr(), n,
                      self.h.data_ptr(), self.scratch.data_ptr(), self.scratch.numel(),
                      None if done is None else done.data_ptr(),
                      torch.cuda.current_stream().cuda_stream), "pbte_arnoldi_column")

    def __del__(self):
        bury(*getattr(self, "graphs", {}).values(), *(getattr(self, "cycle_graphs", None) or {}).values())

    # -- whole restart cycles on the device ----------------------------------
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
        self.tol = torch.zeros(1, **f64)
        self.state = torch.zeros(4, dtype=torch.int32, device=dev)
        self.state_host = torch.zeros(4, dtype=torch.int32, pin_memory=True)
        self.cycle_graphs = {}

    def _cycle_desc(self):
        """The buffers of a cycle with the FP32 product and FP32 basis, for
        ``pbte_gmres_columns_f32`` (which issues a chunk's launches from
        native code); None for the other forms."""
        op = self.op
        if op.precision == "fp64" or self.dtype != torch.float32 or op.per:
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

    def _record_cycle(self, j0: int, j1: int) -> None:
        """Columns j0..j1-1: product, CGS2, rotation, next basis vector; all
        of it skipped once the stop state is set."""
        L = _lib.lib()
        s = torch.cuda.current_stream().cuda_stream
        n, ctx = self.n, self.op.s.ctx.handle
        if self.native_columns:
            if getattr(self, "_desc", None) is None:
                self._desc = self._cycle_desc()
            if self._desc is not None:
                _lib.check(L.pbte_gmres_columns_f32(ctx, ctypes.byref(self._desc), j0, j1, s), "gmres_columns_f32")
                return
        _lib.check(L.pbte_set_done_flag(ctx, self.state.data_ptr()), "set_done_flag")
        try:
            for j in range(j0, j1):
                self._record(j, done=self.state, fill_input=False)
                _lib.check(L.pbte_gmres_givens(j, self.h.data_ptr(), self.R.data_ptr(), self.m_cap,
                                               self.cs.data_ptr(), self.sn.data_ptr(), self.gam.data_ptr(),
                                               self.tol.data_ptr(), self.state.data_ptr(), self.hist.data_ptr(),
                                               s), "gmres_givens")
                nb = L.pbte_gmres_next_basis_f32 if self.dtype == torch.float32 else L.pbte_gmres_next_basis
                _lib.check(nb(j, self.w.data_ptr(), self.h.data_ptr(), self.Q.data_ptr(), self.Q.stride(0),
                              self.op.uin.data_ptr(), n, self.state.data_ptr(), s), "gmres_next_basis")
        finally:
            _lib.check(L.pbte_set_done_flag(ctx, None), "set_done_flag")

    def _chunk(self, j0: int, j1: int):
        key = (j0, j1)
        if key not in self.cycle_graphs:
            if uses_graphs(self.op.s):
                with device_lock:
                    empty_graveyard()
                    torch.cuda.synchronize(self.op.s.device)
                    gr = torch.cuda.CUDAGraph()
                    with torch.cuda.graph(gr, stream=self.stream, capture_error_mode="thread_local"):
                        self._record_cycle(j0, j1)
                self.cycle_graphs[key] = gr
            else:
                return None
        return self.cycle_graphs[key]

    def cycle(self, r: torch.Tensor, beta: float, m: int, tol_abs: float):
        """One restart cycle of at most ``m`` columns from the residual ``r``
        (norm ``beta``), stopping on the device when the residual estimate
        reaches ``tol_abs`` or on breakdown.  Returns ``(k, state, R, gam,
        hist)`` on the host: columns done, stop state (0 none, 1 converged,
        2 breakdown), the k x k triangular factor, the k + 1 residual
        estimates and the k residual norms."""
        self._cycle_buffers()
        n = self.n
        torch.div(r, beta, out=self.Q[0])
        self.op.uin[:n].copy_(self.Q[0])
        self.gam.zero_()
        self.gam[0] = beta
        self.tol.fill_(tol_abs)
        self.state.zero_()
        for j0 in range(0, m, self.CHUNK):
            j1 = min(m, j0 + self.CHUNK)
            g = self._chunk(j0, j1)
            if g is not None:
                g.replay()
            else:
                self._record_cycle(j0, j1)
            self.state_host.copy_(self.state, non_blocking=True)
            torch.cuda.current_stream().synchronize()
            if int(self.state_host[0]) != 0:
                break
        k = int(self.state_host[1])
        R = self.R[:k, :k].cpu().numpy().T.copy()
        gam = self.gam[:k + 1].cpu().numpy()
        hist = self.hist[:k].cpu().numpy()
        self.op.sweeps += k
        if self.on_product is not None:
            for _ in range(k):
                self.on_product()
        return k, int(self.state_host[0]), R, gam, hist

    def _capture(self, j: int) -> None:
        with device_lock:
            empty_graveyard()
            torch.cuda.synchronize(self.op.s.device)
            gr = torch.cuda.CUDAGraph()
            with torch.cuda.graph(gr, stream=self.stream, capture_error_mode="thread_local"):
                self._record(j)
        self.graphs[j] = gr

    def capture_all(self) -> None:
        """Capture every column's graph now (capturing synchronises the
        device, which concurrent solves should not meet mid-run): the
        per-column graphs and the chunks of a full device cycle."""
        for j in range(self.m_cap):
            if j not in self.graphs:
                self._capture(j)
        if self.device_cycles:
            self._cycle_buffers()
            for j0 in range(0, self.m_cap, self.CHUNK):
                self._chunk(j0, min(self.m_cap, j0 + self.CHUNK))

    def column(self, j: int) -> np.ndarray:
        if uses_graphs(self.op.s):
            if j not in self.graphs:
                self._capture(j)
            self.graphs[j].replay()
        else:
            self._record(j)
        self.h_host[:j + 2].copy_(self.h[:j + 2], non_blocking=True)
        torch.cuda.current_stream().synchronize()
        self.op.sweeps += 1
        if self.on_product is not None:
            self.on_product()
        return self.h_host[:j + 2].numpy().copy()


class MomentPreconditioner:
    """Approximate ``(I - T)^-1`` by the GSIS macroscopic system
    (``pybte/krylov.py:369-414``, ``scheme.krylov_precond``): the moment
    blocks of a residual become the source of the HDG local problems, whose
    trace system is solved (with the wall traces of a zero distribution) and
    whose recovered ``T, q_x, q_y`` replace them; the rest of the vector
    passes through.  pybte notes it helps in the diffusive limit and hurts in
    the ballistic one, and leaves it off by default."""

    def __init__(self, solver, acc, sign: float = -1.0, blocks=(0, 1, 2)):
        self.s = solver
        self.acc = acc
        self.nd, self.nt = solver.ndof, solver.n_tris
        self.k = self.nd * self.nt
        self.sign = sign
        self.blocks = blocks
        self.calls = 0
        self.zero_vdf = torch.zeros_like(solver.vdf)
        self.work = torch.zeros((self.nt, 7 * self.nd), dtype=torch.float64, device=solver.device)

    def __call__(self, r: torch.Tensor) -> torch.Tensor:
        a, nd, nt, k = self.acc, self.nd, self.nt, self.k
        self.work.zero_()
        for slot, blk in enumerate(self.blocks):
            if blk is not None:
                self.work[:, blk * nd:(blk + 1) * nd] = self.sign * r[slot * k:(slot + 1) * k].view(nd, nt).T
        aa_src = torch.bmm(a.inv_aa_sol, self.work.unsqueeze(-1)).squeeze(-1).T.contiguous()   # (7nd, n)
        ffa = a.rhs(aa_src, self.zero_vdf)
        u_trace = a.solver.solve(ffa.reshape(-1)).reshape(-1, 3 * a.nf)
        uq = aa_src.T + torch.einsum("ilpr,ilr->ip", a.aa_trace, u_trace[a.tri_faces])              # (n, 7nd)
        out = r.clone()
        out[:3 * k] = uq.T[:3 * nd].reshape(-1)
        self.calls += 1
        return out


def _back_substitute(r, y):
    out = np.array(y, dtype=float)
    for i in range(out.size - 1, -1, -1):
        s = out[i] - r[i, i + 1:] @ out[i + 1:]
        out[i] = s / r[i, i] if r[i, i] != 0.0 else 0.0
    return out


def gmres(matvec, b: torch.Tensor, x0=None, tol_abs: float = 0.0, maxiter=None, max_basis=None,
          callback=None, arnoldi: ArnoldiGraphs | None = None, precond=None):
    """GMRES for ``A x = b`` with device vectors (``pybte/krylov.py:150-246``).
    With ``arnoldi`` (graphs of ``A`` for the same operator) each product and
    its orthogonalisation is one graph replay.  ``precond``: a left
    preconditioner ``M`` (the residuals and products are ``M (b - A x)`` and
    ``M A q``, as pybte's); it takes the host-driven loop.  Returns
    ``(x, converged, n_matvec)``."""
    n = b.numel()
    x = torch.zeros_like(b) if x0 is None else x0.clone()
    maxiter = int(n if maxiter is None else maxiter)
    m_cap = maxiter if max_basis is None else max(1, min(int(max_basis), maxiter))
    if arnoldi is not None and m_cap <= arnoldi.m_cap and precond is None:
        return _gmres_graphs(matvec, b, x, tol_abs, maxiter, m_cap, callback, arnoldi)
    apply_m = (lambda v: v) if precond is None else precond
    nmv = 0
    converged = halted = False
    while nmv < maxiter and not converged and not halted:
        if bool(torch.any(x != 0).item()):
            r = apply_m(b - matvec(x))
            nmv += 1
            if callback is not None and callback(float(torch.linalg.vector_norm(r).item())):
                halted = True
                break
        else:
            r = apply_m(b.clone())
        beta = float(torch.linalg.vector_norm(r).item())
        if beta <= tol_abs:
            converged = True
            break
        m = min(m_cap, maxiter - nmv)
        if m <= 0:
            break
        q = torch.empty((min(m, 64), n), dtype=b.dtype, device=b.device)
        q[0] = r / beta
        cols, cs, sn, gam = [], [], [], [beta]
        for j in range(m):
            w = apply_m(matvec(q[j]))
            nmv += 1
            qj = q[:j + 1]
            c1 = qj @ w
            w -= qj.T @ c1
            c2 = qj @ w
            w -= qj.T @ c2
            hcol = torch.cat([c1 + c2, torch.linalg.vector_norm(w).reshape(1)]).cpu().numpy()
            col = np.array(hcol, dtype=float)
            hn = float(col[j + 1])
            for i in range(j):
                t = cs[i] * col[i] + sn[i] * col[i + 1]
                col[i + 1] = -sn[i] * col[i] + cs[i] * col[i + 1]
                col[i] = t
            d = float(np.hypot(col[j], col[j + 1]))
            c_, s_ = (1.0, 0.0) if d == 0.0 else (col[j] / d, col[j + 1] / d)
            cs.append(c_)
            sn.append(s_)
            col[j] = d
            cols.append(col[:j + 1].copy())
            gam.append(-s_ * gam[j])
            gam[j] = c_ * gam[j]
            res = abs(gam[j + 1])
            stop = bool(callback(res)) if callback is not None else False
            if res <= tol_abs:
                converged = True
                break
            if stop:
                halted = True
                break
            if hn == 0.0:
                break
            if j + 1 < m:
                if j + 1 >= q.shape[0]:
                    grown = torch.empty((min(m, max(2 * q.shape[0], j + 2)), n), dtype=b.dtype, device=b.device)
                    grown[:j + 1] = q[:j + 1]
                    q = grown
                q[j + 1] = w / hn
        k = len(cols)
        if k:
            rmat = np.zeros((k, k))
            for j, col in enumerate(cols):
                rmat[:j + 1, j] = col
            y = torch.from_numpy(_back_substitute(rmat, np.asarray(gam[:k]))).to(b.device)
            x += q[:k].T @ y
    return x, converged, nmv


def _gmres_cycles(matvec, b, x, tol_abs, maxiter, m_cap, ar: ArnoldiGraphs):
    """The loop of :func:`gmres` with whole restart cycles on the device
    (:meth:`ArnoldiGraphs.cycle`): the rotations and the stopping test run
    after each column on the device, the host sees the cycle's end.  Same
    Krylov arithmetic; the rotations use the device's hypot."""
    nmv = 0
    converged = False
    while nmv < maxiter and not converged:
        if bool(torch.any(x != 0).item()):
            r = b - matvec(x)
            nmv += 1
        else:
            r = b.clone()
        beta = float(torch.linalg.vector_norm(r).item())
        if beta <= tol_abs:
            converged = True
            break
        m = min(m_cap, maxiter - nmv)
        if m <= 0:
            break
        k, state, rmat, gam, _ = ar.cycle(r, beta, m, tol_abs)
        nmv += k
        converged = state == 1
        if k:
            y = torch.from_numpy(_back_substitute(rmat, gam[:k])).to(device=b.device, dtype=ar.Q.dtype)
            x += ar.Q[:k].T @ y
    return x, converged, nmv


def _gmres_graphs(matvec, b, x, tol_abs, maxiter, m_cap, callback, ar: ArnoldiGraphs):
    """The loop of :func:`gmres` with the basis in ``ar.Q`` and every Arnoldi
    column from one graph replay; same arithmetic, same stopping."""
    if callback is None and ar.device_cycles:
        return _gmres_cycles(matvec, b, x, tol_abs, maxiter, m_cap, ar)
    nmv = 0
    converged = halted = False
    Q = ar.Q
    while nmv < maxiter and not converged and not halted:
        if bool(torch.any(x != 0).item()):
            r = b - matvec(x)
            nmv += 1
            if callback is not None and callback(float(torch.linalg.vector_norm(r).item())):
                halted = True
                break
        else:
            r = b.clone()
        beta = float(torch.linalg.vector_norm(r).item())
        if beta <= tol_abs:
            converged = True
            break
        m = min(m_cap, maxiter - nmv)
        if m <= 0:
            break
        Q[0].copy_(r / beta)
        cols, cs, sn, gam = [], [], [], [beta]
        for j in range(m):
            col = ar.column(j)
            nmv += 1
            hn = float(col[j + 1])
            for i in range(j):
                t = cs[i] * col[i] + sn[i] * col[i + 1]
                col[i + 1] = -sn[i] * col[i] + cs[i] * col[i + 1]
                col[i] = t
            d = float(np.hypot(col[j], col[j + 1]))
            c_, s_ = (1.0, 0.0) if d == 0.0 else (col[j] / d, col[j + 1] / d)
            cs.append(c_)
            sn.append(s_)
            col[j] = d
            cols.append(col[:j + 1].copy())
            gam.append(-s_ * gam[j])
            gam[j] = c_ * gam[j]
            res = abs(gam[j + 1])
            stop = bool(callback(res)) if callback is not None else False
            if res <= tol_abs:
                converged = True
                break
            if stop:
                halted = True
                break
            if hn == 0.0:
                break
            if j + 1 < m:
                torch.div(ar.w, hn, out=Q[j + 1])
        k = len(cols)
        if k:
            rmat = np.zeros((k, k))
            for j, col in enumerate(cols):
                rmat[:j + 1, j] = col
            y = torch.from_numpy(_back_substitute(rmat, np.asarray(gam[:k]))).to(device=b.device, dtype=Q.dtype)
            x += Q[:k].T @ y
    return x, converged, nmv


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
    if case.scheme.krylov_restart is not None:
        return int(case.scheme.krylov_restart)
    per = max(1.0, 8.0 * float(n))
    return int(max(32, min(int(case.iteration.tmax), int(case.scheme.krylov_max_bytes / per))))


def run_krylov(solver, callback=None, progress_every: int = 0):
    """``pybte/krylov.py:257-363`` on the device.  ``callback(step,
    residual, solver)`` and progress lines follow every residual the host
    sees (each product's GMRES residual, the closing true residual); a
    restarted solver starts GMRES from its loaded state."""
    c = solver.case
    tol, tmax = c.iteration.tol, c.iteration.tmax
    want_true = c.iteration.true_residual
    op = cached(solver, "fp64", lambda: FixedPointOperator(solver))
    op.sweeps = 0
    residuals, masses, true_res = [], [], []

    def sweep(u):
        out = op.apply(u)
        product()
        return out

    def product():
        masses.append(np.nan)
        residuals.append(np.nan)
        if want_true:
            true_res.append(np.nan)

    def close(res):
        residuals[-1] = res
        step = len(residuals)
        if progress_every and step % progress_every == 0:
            print(f"  step {step:8d}  residual {res:.6e}", flush=True)
        if callback is not None:
            callback(step, res, solver)

    sync(solver.device)
    t0 = time.perf_counter()
    restarted = bool(solver.restart_info.get("enabled")) if hasattr(solver, "restart_info") else False
    x = op.state() if restarted else torch.zeros(op.n, dtype=torch.float64, device=solver.device)
    zero = torch.zeros(op.n, dtype=torch.float64, device=solver.device)
    g = sweep(zero)
    gnorm = float(torch.linalg.vector_norm(g).item())
    scale = gnorm or 1.0
    close(1.0)

    def matvec(v):
        return v - (sweep(v) - g)

    enough = max(tol * _ENOUGH, _FLOOR) * scale
    target = max(tol * c.scheme.krylov_tol_factor, _FLOOR) * scale
    cap = basis_cap(c, op.n)
    reached = -1

    def on_residual(res):
        nonlocal reached
        close(res / scale)
        n = len(residuals)
        if reached < 0 and res <= enough:
            reached = n
        return reached >= 0 and n - reached > max(64, reached // 4)

    precond = None
    if c.scheme.krylov_precond and getattr(solver, "acc", None) is not None:
        precond = MomentPreconditioner(solver, solver.acc)
    ar = (cached(solver, ("arnoldi64", cap), lambda: ArnoldiGraphs(op, g, cap))
          if cap <= 63 and precond is None else None)
    if ar is not None:
        ar.set_g(g)
        ar.on_product = product
    converged = False
    final = float("nan")
    for _ in range(c.scheme.krylov_max_rounds):
        budget = tmax - len(residuals) - 1
        if budget <= 0:
            break
        reached = -1
        x, _, _ = gmres(matvec, g, x0=x, tol_abs=target, maxiter=budget, max_basis=cap, callback=on_residual,
                        arnoldi=ar, precond=precond)
        sweep(x)
        op.publish()
        final = solver.ctx.true_residual(solver.mom, solver.vdf)
        if want_true:
            true_res[-1] = final
        close(final)
        converged = bool(final < tol) if np.isfinite(final) else gnorm == 0.0
        if converged or len(residuals) >= tmax:
            break
        target = max(target * 1.0e-3, _FLOOR * scale)
    sync(solver.device)
    wall = time.perf_counter() - t0
    solver.ctx.sweep_count += op.sweeps
    masses = [solver.mom.mass] * len(residuals)
    return solver._record(len(residuals), converged, residuals, masses, wall, "KRYLOV",
                          extra={"krylov_size": op.n, "krylov_periodic_state": op.nper, "krylov_basis_cap": cap,
                                 "krylov_precond": precond is not None, "transport_residual": final},
                          true_res=true_res if want_true else None)
