"""GSIS / HDG macroscopic acceleration on the device (``pybte/acceleration/``).

Per outer iteration, after the sweep (``acceleration/__init__.py:95-115``):

1. hot source: third-order angular moments of the kinetic solution contracted
   with the gradient tensors and premultiplied by the element inverses
   ``inv_aa_sol`` (``pbte_gsis_hot_apply``: one angular-sum launch, then one
   launch that forms each element's source in shared memory and applies the
   inverse);
2. trace right-hand side: ``BA_SOL @ AA_SRC`` from the one or two elements of
   each face, wall rows imposed from the kinetic wall traces
   (``pbte_wall_trace``, ``pbte_gsis_trace_rhs``);
3. trace solve with the once-factorised global matrix: on the device from
   nested-dissection multifrontal factors (:mod:`pbte_gb300.trace_nd`,
   default), or SuperLU on the host (``performance.trace_solver = "host"``);
4. local recovery ``UQ = AA_SRC + sum AA_TRACE @ U_TRACE``
   (``pbte_gsis_local_recover``);
5. damped correction of the distribution and the moments (``pbte_correct``).

Every per-iteration launch is the library's own kernel; the element and face
operators are stored field-major (``pbte_gsis_ops``) so that each of those
kernels reads them coalesced.  With the device trace solve, a GSIS step is
graph-captured and every launch honours the run's device stop flag.

Setup (``assembly.py:44-269``) builds the 7x7-block element matrices on the
host, inverts them with the library's batched Gauss-Jordan kernel, forms
``AA_TRACE``, ``BA_SOL`` and the sparse trace matrix, and factorises it once.
The defect-repair experiment of the reference (off by default there) is not
carried.
"""
from __future__ import annotations

import ctypes

import numpy as np
import torch

from . import _lib
from .device import bury, device_lock, empty_graveyard
from .constants import BC_NONTHERMALISING, BC_PERIODIC, BC_THERMALISING
from .trace_nd import NestedDissectionSolver
from .trace_solver import TraceSolver

__all__ = ["GSIS", "GsisFixedPoint", "local_blocks"]


def _mirror_perm(nf):
    base = np.arange(nf)[::-1]
    return np.concatenate([base + b * nf for b in range(3)])


def local_blocks(disc, st, variant):
    """Element matrices ``AA_SOL`` (n, 7nd, 7nd) and trace couplings ``T``
    (n, 3, 7nd, 3nf) of ``build_local_operators`` (``assembly.py:44-125``)."""
    c, m, it = disc.case, disc.mesh, disc.integrals
    nd, nf = disc.ndof, c.ndof_fc
    n = m.n_tris
    tau_r, tau_c, cv = c.flow.tau_r, c.tau_c, c.flow.cv
    scale = tau_r if variant == "B" else 1.0
    aa, bb = it.int_tri_tri_x, it.int_tri_tri_y
    cc, dd = np.transpose(aa, (0, 2, 1)), np.transpose(bb, (0, 2, 1))
    pp = it.int_tri_fc.sum(axis=1)
    oo = np.transpose(it.int_tri_tri, (2, 0, 1))
    A = np.zeros((n, 7 * nd, 7 * nd))

    def put(r, col, v):
        A[:, r * nd:(r + 1) * nd, col * nd:(col + 1) * nd] = v
    put(0, 0, st[0] * pp); put(0, 1, cc); put(0, 2, dd)
    put(1, 0, -aa * cv / 3.0 * scale)
    put(1, 1, (oo + st[1] * pp) if variant == "B" else (st[1] * pp + oo / tau_r))
    put(1, 3, -4.0 / 3.0 * cc); put(1, 4, -dd); put(1, 5, -dd); put(1, 6, 2.0 / 3.0 * cc)
    put(2, 0, -bb * cv / 3.0 * scale)
    put(2, 2, (oo + st[2] * pp) if variant == "B" else (st[2] * pp + oo / tau_r))
    put(2, 3, 2.0 / 3.0 * dd); put(2, 4, -cc); put(2, 5, -cc); put(2, 6, -4.0 / 3.0 * dd)
    tc5 = tau_c * scale / 5.0
    put(3, 1, aa * tc5); put(3, 3, oo); put(4, 1, bb * tc5); put(4, 4, oo)
    put(5, 2, aa * tc5); put(5, 5, oo); put(6, 2, bb * tc5); put(6, 6, oo)

    ww = np.transpose(it.int_tri_fc_fc, (2, 3, 0, 1))           # (n, 3, nd, nf)
    nxe = m.tri_normal[:, :, 0][:, :, None, None]
    nye = m.tri_normal[:, :, 1][:, :, None, None]
    T = np.zeros((n, 3, 7 * nd, 3 * nf))

    def tput(r, col, v):
        T[:, :, r * nd:(r + 1) * nd, col * nf:(col + 1) * nf] = v
    tput(0, 0, st[0] * ww)
    tput(1, 0, -nxe * ww * cv / 3.0 * scale); tput(1, 1, st[1] * ww)
    tput(2, 0, -nye * ww * cv / 3.0 * scale); tput(2, 2, st[2] * ww)
    tput(3, 1, nxe * ww * tc5); tput(4, 1, nye * ww * tc5)
    tput(5, 2, nxe * ww * tc5); tput(6, 2, nye * ww * tc5)
    return A, T, tc5


def ba_sol_blocks(disc, st, variant):
    """``BA_SOL`` (n, 3, 3nf, 7nd) of ``build_ba_sol`` (``assembly.py:128-184``)."""
    c, m, it = disc.case, disc.mesh, disc.integrals
    nd, nf = disc.ndof, c.ndof_fc
    bc_type = disc.bcdata.bc_type
    B = np.zeros((m.n_tris, 3, 3 * nf, 7 * nd))
    bb2 = np.transpose(it.int_tri_fc_fc, (2, 3, 1, 0))
    nx = m.tri_normal[:, :, 0][:, :, None, None]
    ny = m.tri_normal[:, :, 1][:, :, None, None]
    fb = m.face_bc[m.tri_faces]
    code = np.where(fb >= 0, bc_type[np.clip(fb, 0, None)], 0)
    interior = fb < 0
    std = (interior | ((~interior) & (code == BC_PERIODIC)))[:, :, None, None]
    wall_th = ((~interior) & (code == BC_THERMALISING))[:, :, None, None]

    std_f = std.astype(float)
    wall_f = wall_th.astype(float)

    def put(r, col, v, mask):
        # the two masks are disjoint and every block starts at zero, so a
        # masked add is the masked assignment
        sl = (slice(None), slice(None), slice(r * nf, (r + 1) * nf), slice(col * nd, (col + 1) * nd))
        B[sl] += v * (std_f if mask is std else wall_f)
    put(0, 0, 0.5 * bb2, std); put(0, 1, nx / 2.0 / st[0] * bb2, std); put(0, 2, ny / 2.0 / st[0] * bb2, std)
    put(1, 1, 0.5 * bb2, std); put(1, 3, -2.0 * nx / 3.0 / st[1] * bb2, std)
    put(1, 4, -ny / 2.0 / st[1] * bb2, std); put(1, 5, -ny / 2.0 / st[1] * bb2, std)
    put(1, 6, nx / 3.0 / st[1] * bb2, std)
    put(2, 2, 0.5 * bb2, std); put(2, 3, ny / 3.0 / st[2] * bb2, std)
    put(2, 4, -nx / 2.0 / st[2] * bb2, std); put(2, 5, -nx / 2.0 / st[2] * bb2, std)
    put(2, 6, -2.0 * ny / 3.0 / st[2] * bb2, std)
    if variant == "A":
        put(1, 1, bb2, wall_th); put(1, 3, -4.0 * nx / 3.0 / st[1] * bb2, wall_th)
        put(1, 4, -ny / st[1] * bb2, wall_th); put(1, 5, -ny / st[1] * bb2, wall_th)
        put(1, 6, 2.0 * nx / 3.0 / st[1] * bb2, wall_th)
        put(2, 2, bb2, wall_th); put(2, 3, 2.0 * ny / 3.0 / st[2] * bb2, wall_th)
        put(2, 4, -nx / st[2] * bb2, wall_th); put(2, 5, -nx / st[2] * bb2, wall_th)
        put(2, 6, -4.0 * ny / 3.0 / st[2] * bb2, wall_th)
    return B


class GSIS:
    def __init__(self, solver):
        from scipy.sparse import coo_matrix

        s = solver
        disc = s.disc
        c, m, it = disc.case, disc.mesh, disc.integrals
        self.s = s
        dev = s.device
        nd, nf = disc.ndof, c.ndof_fc
        self.nd, self.nf = nd, nf
        self.variant = c.scheme.acc_variant
        if c.scheme.defect_omega != 0.0 or c.scheme.defect_anderson:
            raise NotImplementedError("scheme.defect_omega / defect_anderson (pybte's experimental defect "
                                      "repair, off by default there) are not implemented")
        st = np.asarray(c.scheme.stabilisation, dtype=float).copy()
        if c.scheme.scale_by_hmin:
            st[1] /= m.hmin
            st[2] /= m.hmin
        self.st = st
        n = m.n_tris
        A, T, self.tc5 = local_blocks(disc, st, self.variant)
        f64 = dict(dtype=torch.float64, device=dev)
        A_d = torch.from_numpy(A).to(dev)
        inv = torch.empty_like(A_d)
        bad = torch.zeros(1, dtype=torch.int32, device=dev)
        _lib.check(_lib.lib().pbte_batched_inverse(A_d.data_ptr(), inv.data_ptr(), n, 7 * nd, bad.data_ptr(),
                                                   torch.cuda.current_stream().cuda_stream), "batched_inverse")
        if int(bad.item()):
            raise np.linalg.LinAlgError(f"{int(bad.item())} singular HDG element matrices")
        del A_d
        T_d = torch.from_numpy(T).to(dev)
        aa_trace = torch.einsum("ipq,ilqr->ilpr", inv, T_d).contiguous()   # (n, 3, 7nd, 3nf)
        del T_d
        # field-major copies for the per-iteration kernels (pbte_gsis_ops)
        self.inv_t = inv.permute(2, 0, 1).contiguous()                   # [q][i][p] = inv[i][p][q]
        self.aa_trace_t = aa_trace.permute(1, 3, 0, 2).contiguous()      # [il][r][i][p]
        self.aa_trace = aa_trace
        del inv
        B = ba_sol_blocks(disc, st, self.variant)
        self.ba_sol = torch.from_numpy(B).to(dev)                        # (n, 3, 3nf, 7nd)

        bc_type = disc.bcdata.bc_type
        flip = disc.bcdata.periodic_flip
        perm = _mirror_perm(nf)
        nf3 = 3 * nf
        adj_t, adj_l = m.adjacent_all()
        fbc = m.face_bc
        code = np.where(fbc >= 0, bc_type[np.clip(fbc, 0, None)], 0)
        interior = fbc < 0
        periodic = (~interior) & (code == BC_PERIODIC)
        p1_tri = np.where(interior, m.face_tri[:, 0], adj_t).astype(np.int64)
        p1_lfc = np.where(interior, m.face_lfc[:, 0], adj_l).astype(np.int64)
        p2_tri = np.full(m.n_faces, -1, dtype=np.int64)
        p2_lfc = np.full(m.n_faces, -1, dtype=np.int64)
        p2_tri[interior] = m.face_tri[interior, 1]
        p2_lfc[interior] = m.face_lfc[interior, 1]
        if periodic.any():
            pf = np.flatnonzero(periodic)
            p2_tri[pf] = adj_t[m.face_pair[pf]]
            p2_lfc[pf] = adj_l[m.face_pair[pf]]
        has_p2 = p2_tri >= 0
        mirror2 = periodic & flip

        # global trace matrix K (assembly.py:200-269), blocks formed on the device
        rows, cols, vals = [], [], []
        diag = np.zeros((m.n_faces, nf3, nf3))
        for k in range(3):
            diag[:, k * nf:(k + 1) * nf, k * nf:(k + 1) * nf] = np.transpose(it.int_fc_fc, (2, 0, 1))
        rr, cc = np.meshgrid(np.arange(nf3), np.arange(nf3), indexing="ij")
        fid = np.arange(m.n_faces)
        rows.append((fid[:, None, None] * nf3 + rr).ravel())
        cols.append((fid[:, None, None] * nf3 + cc).ravel())
        vals.append(diag.ravel())
        permt = torch.from_numpy(perm).to(dev)
        for side in (0, 1):
            sel = np.ones(m.n_faces, bool) if side == 0 else has_p2
            fsel = np.flatnonzero(sel)
            tri = (p1_tri if side == 0 else p2_tri)[fsel]
            lfc = (p1_lfc if side == 0 else p2_lfc)[fsel]
            ba = self.ba_sol[torch.from_numpy(tri).to(dev), torch.from_numpy(lfc).to(dev)]       # (k, nf3, 7nd)
            for il in range(3):
                at = self.aa_trace[torch.from_numpy(tri).to(dev), il]                                  # (k, 7nd, nf3)
                D = torch.bmm(ba, at)
                if side == 1 and mirror2[fsel].any():
                    mm = torch.from_numpy(mirror2[fsel]).to(dev)
                    D[mm] = D[mm][:, permt]
                g = m.tri_faces[tri, il]
                rows.append((fsel[:, None, None] * nf3 + rr).ravel())
                cols.append((g[:, None, None] * nf3 + cc).ravel())
                vals.append((-D).cpu().numpy().ravel())
        nn = m.n_faces * nf3
        K = coo_matrix((np.concatenate(vals), (np.concatenate(rows), np.concatenate(cols))),
                       shape=(nn, nn)).tocsr()
        K.sum_duplicates()
        drop = 1e-30 if self.variant == "A" else 0.0
        K.data[np.abs(K.data) <= drop] = 0.0
        K.eliminate_zeros()
        K.sort_indices()
        self.K = K
        if c.performance.trace_solver == "device":
            xy = m.nodes[m.face_nodes].mean(axis=1)
            self.solver = NestedDissectionSolver(K, xy, nf3, dev)
        else:
            self.solver = TraceSolver(K, dev)

        # per-iteration operators (global_solve.py:88-117), field-major
        i32 = dict(dtype=torch.int32, device=dev)
        sel2 = np.flatnonzero(has_p2)
        ba1 = self.ba_sol[torch.from_numpy(p1_tri).to(dev), torch.from_numpy(p1_lfc).to(dev)]   # (n_faces, nf3, 7nd)
        self.ba1_t = ba1.permute(2, 0, 1).contiguous()                                          # [p][f][r]
        del ba1
        self.n2 = int(sel2.size)
        if self.n2:
            ba2 = self.ba_sol[torch.from_numpy(p2_tri[sel2]).to(dev), torch.from_numpy(p2_lfc[sel2]).to(dev)]
            self.ba2_t = ba2.permute(2, 0, 1).contiguous()
            del ba2
        else:
            self.ba2_t = torch.zeros(1, **f64)
        del self.ba_sol, self.aa_trace
        slot2 = np.full(m.n_faces, -1, dtype=np.int32)
        slot2[sel2] = np.arange(self.n2, dtype=np.int32)
        self.tri1 = torch.from_numpy(p1_tri.astype(np.int32)).to(dev)
        self.slot2 = torch.from_numpy(slot2).to(dev)
        self.tri2 = torch.from_numpy(p2_tri[sel2].astype(np.int32)).to(dev) if self.n2 else torch.zeros(1, **i32)
        self.mirror2 = (torch.from_numpy(mirror2[sel2].astype(np.int32)).to(dev) if self.n2
                        else torch.zeros(1, **i32))
        wall_th = np.flatnonzero((fbc >= 0) & (code == BC_THERMALISING))
        wall_ad = np.flatnonzero((fbc >= 0) & (code == BC_NONTHERMALISING))
        self.wall_all = np.concatenate([wall_th, wall_ad])
        self.n_th = wall_th.size
        wall_slot = np.full(m.n_faces, -1, dtype=np.int32)
        wall_slot[self.wall_all] = np.arange(self.wall_all.size, dtype=np.int32)
        wall_kind = np.zeros(m.n_faces, dtype=np.int32)
        wall_kind[wall_th] = 1
        wall_kind[wall_ad] = 2
        self.wall_slot = torch.from_numpy(wall_slot).to(dev)
        self.wall_kind = torch.from_numpy(wall_kind).to(dev)
        self.wall_nx = torch.from_numpy(np.ascontiguousarray(m.tri_normal[p1_tri, p1_lfc, 0])).to(dev)
        self.wall_ny = torch.from_numpy(np.ascontiguousarray(m.tri_normal[p1_tri, p1_lfc, 1])).to(dev)
        self.wall_tri = torch.from_numpy(p1_tri[self.wall_all].astype(np.int32)).to(dev)
        self.wall_lfc = torch.from_numpy(p1_lfc[self.wall_all].astype(np.int32)).to(dev)
        self.tri_fc_fc = torch.from_numpy(np.ascontiguousarray(it.int_tri_fc_fc)).to(dev)
        self.tri_faces = torch.from_numpy(m.tri_faces.astype(np.int32)).to(dev)
        self.tri_hmin = torch.from_numpy(np.ascontiguousarray(m.tri_hmin)).to(dev)
        self.use_hmin = self.variant == "A"
        self.ops = _lib.GsisOps(
            n, m.n_faces, nd, nf, 1 if self.variant == "B" else 0, self.n2, int(self.wall_all.size), 0, c.flow.cv,
            self.inv_t.data_ptr(), self.ba1_t.data_ptr(), self.tri1.data_ptr(), self.ba2_t.data_ptr(),
            self.slot2.data_ptr(), self.tri2.data_ptr(), self.mirror2.data_ptr(), self.wall_slot.data_ptr(),
            self.wall_kind.data_ptr(), self.wall_nx.data_ptr(), self.wall_ny.data_ptr(),
            self.aa_trace_t.data_ptr(), self.tri_faces.data_ptr())
        self.aa_src = torch.zeros((n, 7 * nd), **f64)
        self.wall_mom = torch.zeros((max(1, self.wall_all.size), nf3), **f64)
        self.ffa = torch.zeros((m.n_faces, nf3), **f64)
        self.u_trace = torch.zeros(m.n_faces * nf3, **f64)
        self.uq = torch.zeros((7 * nd, n), **f64)
        #: the run's device stop flag (int32 tensor) while a device-stopped
        #: loop is captured: every launch of the step then returns at once
        #: once it is set
        self.done = None
        self.solve_count = 0
        #: host bytes this setup moved to the device (the element and face
        #: blocks and the trace matrix the factorisation starts from)
        self.h2d_bytes = int(A.nbytes + T.nbytes + B.nbytes + K.data.nbytes + K.indices.nbytes + K.indptr.nbytes)

    def diagnostics(self) -> dict:
        """The run-record entries of ``Acceleration.diagnostics``
        (``pybte/acceleration/__init__.py:175-187``); the defect-repair
        experiment is not implemented, so its entries are its off values."""
        return {"acc_variant": self.variant, "global_matrix_n": int(self.K.shape[0]),
                "global_matrix_nnz": int(self.K.nnz), "global_solve_count": int(self.solve_count),
                "stabilisation": [float(v) for v in self.st], "defect_omega": 0.0, "defect_every": 1,
                "defect_anderson": 0, "defect_outer": 0, "defect_norm": 0.0}

    def _done_ptr(self):
        return None if self.done is None else self.done.data_ptr()

    def rhs(self, aa_src: torch.Tensor, vdf: torch.Tensor, stream=None) -> torch.Tensor:
        """``GlobalSolver.rhs`` (``global_solve.py:131-187``) into ``self.ffa``
        (n_faces, 3nf): ``aa_src`` is (n_tris, 7nd), element-major."""
        L = _lib.lib()
        s = (stream or torch.cuda.current_stream()).cuda_stream
        if self.wall_all.size:
            _lib.check(L.pbte_wall_trace(self.s.ctx.handle, vdf.data_ptr(), self.tri_fc_fc.data_ptr(),
                                         int(self.wall_all.size), self.wall_tri.data_ptr(),
                                         self.wall_lfc.data_ptr(), self.wall_mom.data_ptr(), s), "wall_trace")
        _lib.check(L.pbte_gsis_trace_rhs(ctypes.byref(self.ops), aa_src.data_ptr(), self.wall_mom.data_ptr(),
                                         self.ffa.data_ptr(), self._done_ptr(), s), "gsis_trace_rhs")
        return self.ffa

    def trace_solve(self, stream=None) -> torch.Tensor:
        """The trace unknowns from ``self.ffa`` into ``self.u_trace``."""
        if isinstance(self.solver, NestedDissectionSolver):
            self.solver.solve(self.ffa.view(-1), out=self.u_trace, stream=stream, done=self.done)
        else:
            self.u_trace.copy_(self.solver.solve(self.ffa.view(-1)))
        return self.u_trace

    def recover(self, aa_src: torch.Tensor, out: torch.Tensor, stream=None) -> torch.Tensor:
        """``local_solve`` (``local_solve.py:16-26``): ``out`` (7nd, n_tris)
        from ``aa_src`` and the current trace unknowns."""
        s = (stream or torch.cuda.current_stream()).cuda_stream
        _lib.check(_lib.lib().pbte_gsis_local_recover(ctypes.byref(self.ops), aa_src.data_ptr(),
                                                      self.u_trace.data_ptr(), out.data_ptr(), self._done_ptr(), s),
                   "gsis_local_recover")
        return out

    def apply(self, stream=None) -> None:
        s = self.s
        L = _lib.lib()
        st = (stream or torch.cuda.current_stream()).cuda_stream
        _lib.check(L.pbte_gsis_hot_apply(s.ctx.handle, ctypes.byref(self.ops), s.vdf.data_ptr(), float(self.tc5),
                                         self.aa_src.data_ptr(), st), "gsis_hot_apply")
        self.rhs(self.aa_src, s.vdf, stream)
        self.trace_solve(stream)
        self.solve_count += 1
        self.recover(self.aa_src, self.uq, stream)
        m = s.mom
        _lib.check(L.pbte_correct(s.ctx.handle, s.vdf.data_ptr(), self.uq.data_ptr(), self.tri_hmin.data_ptr(),
                                  float(s.case.flow.tau_thr), int(self.use_hmin), m.ts.data_ptr(),
                                  m.qxs.data_ptr(), m.qys.data_ptr(), m.temp.data_ptr(), m.qx.data_ptr(),
                                  m.qy.data_ptr(), st), "correct")


class GsisFixedPoint:
    """One GSIS iteration as an affine map ``u -> G(u)`` on the sweep's inputs
    ``u = [ts, qxs, qys, flux_wall]`` (the moment sources, then the adiabatic
    wall emission when there are adiabatic walls): sweep, then the whole
    acceleration step (``acceleration/__init__.py:95-115``), then the new
    moments and the emission of the corrected distribution.  Its fixed point
    is the GSIS solver's (``Solver.step`` iterates exactly this map), so the
    mixed-precision solve can refine it in FP64 around FP32 products.

    ``precision="fp64"``: the FP64 drop-in's kernels on the solver's
    distribution.  ``precision="fp32"`` (homogeneous only: the walls' fixed
    temperatures dropped, the map's linear part): the folded FP32 sweep and
    the FP32 GSIS kernels on an FP32 distribution with FP32 angular sums; the
    trace right-hand side, the trace solve and the local recovery stay FP64.
    The interface is :class:`pbte_gb300.krylov.FixedPointOperator`'s."""

    native_product = False   # no fused native GMRES chunks for this product

    def __init__(self, solver, precision: str = "fp64", homogeneous: bool = False):
        s = solver
        if s.acc is None:
            raise ValueError("GsisFixedPoint needs a solver with the GSIS acceleration")
        if s.bcdata.has_periodic:
            raise NotImplementedError("mixed-precision GSIS with periodic faces")
        if precision == "fp32" and not homogeneous:
            raise ValueError("the FP32 GSIS product is the homogeneous map only")
        self.s = s
        self.acc = s.acc
        self.nd, self.nt = s.ndof, s.n_tris
        self.k = self.nd * self.nt
        self.nmom = 3 * self.k
        self.wall = bool(s.bcdata.has_nonthermalising)
        self.nwall = s.mesh.n_faces * self.nd if self.wall else 0
        self.per = False
        self.nper = 0
        self.n = self.nmom + self.nwall
        self.precision = precision
        self.homogeneous = homogeneous
        self.integrals = True
        dev = s.device
        f64 = dict(dtype=torch.float64, device=dev)
        self.uin = torch.zeros(self.n, **f64)
        self.uout = torch.zeros_like(self.uin)
        self.temp = torch.zeros(self.nt, **f64)
        self.qx = torch.zeros(self.nt, **f64)
        self.qy = torch.zeros(self.nt, **f64)
        if precision == "fp64":
            self.vdf = s.vdf
        else:
            self.vdf = torch.zeros((s.ctx.schedule()["unique_dirs"], self.nt, self.nd), dtype=torch.float32,
                                   device=dev)
            self.uq = torch.zeros_like(self.acc.uq)
            self.scratch_mom = torch.zeros((3, self.nd, self.nt), **f64)
        self.sweeps = 0
        self.graph = None
        self.stream = torch.cuda.Stream(device=dev)

    def _views(self, u):
        k, m = self.k, self.nmom
        fw = u[m:m + self.nwall].view(-1, self.nd) if self.wall else None
        return (u[:k].view(self.nd, self.nt), u[k:2 * k].view(self.nd, self.nt),
                u[2 * k:3 * k].view(self.nd, self.nt), fw, None)

    @staticmethod
    def _ptr(t):
        return t.data_ptr() if t is not None else None

    def _launch(self, st: int, done=None) -> None:
        L = _lib.lib()
        s, a = self.s, self.acc
        ctx = s.ctx.handle
        ts, qxs, qys, fw, _ = self._views(self.uin)
        ots, oqxs, oqys, ofw, _ = self._views(self.uout)
        fw_in = fw if fw is not None else s.ctx.flux_wall
        # the stream whose handle is st is the current one (direct launches,
        # or the capturing stream); a stream object is not rebuilt from the
        # handle, since torch maps a null handle to a new pool stream
        stream = torch.cuda.current_stream(s.device)
        if stream.cuda_stream != st:
            raise RuntimeError("GsisFixedPoint launches on the current stream only")
        keep, a.done = a.done, done
        try:
            if self.precision == "fp64":
                _lib.check(L.pbte_sweep(ctx, ts.data_ptr(), qxs.data_ptr(), qys.data_ptr(), self.vdf.data_ptr(),
                                        fw_in.data_ptr(), s.ctx.pbuf.data_ptr(), 0, st), "sweep")
                _lib.check(L.pbte_gsis_hot_apply(ctx, ctypes.byref(a.ops), self.vdf.data_ptr(), float(a.tc5),
                                                 a.aa_src.data_ptr(), st), "gsis_hot_apply")
                a.rhs(a.aa_src, self.vdf, stream)
                a.trace_solve(stream)
                a.recover(a.aa_src, a.uq, stream)
                _lib.check(L.pbte_correct(ctx, self.vdf.data_ptr(), a.uq.data_ptr(), a.tri_hmin.data_ptr(),
                                          float(s.case.flow.tau_thr), int(a.use_hmin), ots.data_ptr(),
                                          oqxs.data_ptr(), oqys.data_ptr(), self.temp.data_ptr(), self.qx.data_ptr(),
                                          self.qy.data_ptr(), st), "correct")
                if self.wall:
                    _lib.check(L.pbte_wall_flux(ctx, self.vdf.data_ptr(), ofw.data_ptr(), st), "wall_flux")
                return
            _lib.check(L.pbte_sweep_fold_f32(ctx, ts.data_ptr(), qxs.data_ptr(), qys.data_ptr(), fw_in.data_ptr(),
                                             0.0 if self.homogeneous else 1.0, self.vdf.data_ptr(), st),
                       "sweep_fold_f32")
            self._after_sweep32(st, stream)
        finally:
            a.done = keep

    def batch_item(self, done=None) -> "_lib.BatchItem":
        """The FP32 product's sweep as an item of a batched sweep
        (``pbte_sweep_batch_*``)."""
        if self.precision != "fp32":
            raise ValueError("only the FP32 product sweeps in a batch")
        ts, qxs, qys, fw, _ = self._views(self.uin)
        fw_in = fw if fw is not None else self.s.ctx.flux_wall
        return _lib.BatchItem(self.s.ctx.handle.value, ts.data_ptr(), qxs.data_ptr(), qys.data_ptr(),
                              fw_in.data_ptr(), 0.0 if self.homogeneous else 1.0, self.vdf.data_ptr(),
                              None if done is None else done.data_ptr())

    def after_sweep(self, st: int, done=None) -> None:
        """The FP32 product's launches after a batched sweep (the GSIS chain)."""
        a = self.acc
        keep, a.done = a.done, done
        try:
            self._after_sweep32(st, torch.cuda.current_stream(self.s.device))
        finally:
            a.done = keep

    def _after_sweep32(self, st: int, stream) -> None:
        L = _lib.lib()
        s, a = self.s, self.acc
        ctx = s.ctx.handle
        ots, oqxs, oqys, ofw, _ = self._views(self.uout)
        v = self.vdf.data_ptr()
        _lib.check(L.pbte_gsis_hot_apply_f32(ctx, ctypes.byref(a.ops), v, float(a.tc5), a.aa_src.data_ptr(), st),
                   "gsis_hot_apply_f32")
        if a.wall_all.size:
            _lib.check(L.pbte_wall_trace_f32(ctx, v, a.tri_fc_fc.data_ptr(), int(a.wall_all.size),
                                             a.wall_tri.data_ptr(), a.wall_lfc.data_ptr(), a.wall_mom.data_ptr(),
                                             st), "wall_trace_f32")
        _lib.check(L.pbte_gsis_trace_rhs(ctypes.byref(a.ops), a.aa_src.data_ptr(), a.wall_mom.data_ptr(),
                                         a.ffa.data_ptr(), a._done_ptr(), st), "gsis_trace_rhs")
        a.trace_solve(stream)
        a.recover(a.aa_src, self.uq, stream)
        # the new moments are the distribution's plus the damped corrections
        # (correction.py: not the moments of the corrected distribution,
        # whose flux part differs by tau_C / tau_N); the emission is the
        # corrected distribution's
        _lib.check(L.pbte_correct_f32(ctx, v, self.uq.data_ptr(), a.tri_hmin.data_ptr(),
                                      float(s.case.flow.tau_thr), int(a.use_hmin), ots.data_ptr(),
                                      oqxs.data_ptr(), oqys.data_ptr(), st), "correct_f32")
        if self.wall:
            m = self.scratch_mom
            _lib.check(L.pbte_fold_epilogue_f32(ctx, v, m[0].data_ptr(), m[1].data_ptr(), m[2].data_ptr(),
                                                ofw.data_ptr(), None, None, None, st), "fold_epilogue_f32")

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
        """G(u), stream-ordered on the current stream."""
        self.uin.copy_(u)
        if getattr(self.s, "use_graphs", True) and self.s.case.performance.trace_solver == "device":
            if self.graph is None:
                self._capture()
            self.graph.replay()
        else:
            self._launch(torch.cuda.current_stream().cuda_stream)
        self.sweeps += 1
        return self.uout.clone()

    def state(self) -> torch.Tensor:
        """The state of the solver's current distribution and moments (a
        restart's start): the moments, and the wall emission of ``vdf``."""
        s = self.s
        u = torch.zeros_like(self.uin)
        ts, qxs, qys, fw, _ = self._views(u)
        ts.copy_(s.mom.ts)
        qxs.copy_(s.mom.qxs)
        qys.copy_(s.mom.qys)
        if self.wall:
            s.ctx.wall_flux(s.vdf, out=fw)
        return u

    def publish(self) -> None:
        """The last product's moments and emission into the solver's state."""
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
