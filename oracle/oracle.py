"""TEST INFRASTRUCTURE ONLY -- the CPU oracle for the GPU path.

A restatement of the reference solver's hot path (dingtao-shen/...-PBTE,
``solver-python/pybte``): the transport sweep, moments, residuals and wall
emission in plain C (``pbte_oracle.c``, statement-for-statement with
``pybte/_kernels.py``), and the three outer iterations in Python/numpy:

* CIS source iteration      -- ``pybte/driver.py:149-215``
* GMRES on the fixed point  -- ``pybte/krylov.py:64-363`` (CGS2, Givens)
* GSIS / HDG acceleration   -- ``pybte/acceleration/*.py``

It consumes the setup arrays of a :class:`pbte_gb300.discretisation.Discretisation`
(the setup itself is pinned against pybte by the golden fixtures).  Only the
tests, ``__graft_entry__.smoke`` and ``bench.py``'s CPU-baseline leg use this
module; the product never imports it.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
import time
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB = HERE / "_build" / "libpbte_oracle.so"
PI = 4.0 * np.arctan(1.0)

_d = ctypes.POINTER(ctypes.c_double)
_i = ctypes.POINTER(ctypes.c_int)


class OrcCtx(ctypes.Structure):
    _fields_ = [("ndir", ctypes.c_int), ("n_tris", ctypes.c_int), ("nd", ctypes.c_int),
                ("n_faces", ctypes.c_int), ("nbc", ctypes.c_int), ("order", _i),
                ("cxv", _d), ("cyv", _d), ("domega", _d),
                ("cv", ctypes.c_double), ("vg", ctypes.c_double), ("tau_r", ctypes.c_double),
                ("tau_n", ctypes.c_double), ("tau_c", ctypes.c_double), ("pi", ctypes.c_double),
                ("mass", _d), ("gx", _d), ("gy", _d), ("fcm", _d), ("ttfc", _d),
                ("nx", _d), ("ny", _d), ("tri_faces", _i), ("face_bc", _i),
                ("neighbour", _i), ("periodic_tri", _i), ("bc_type", _i),
                ("bc_temp", _d), ("flux_wall", _d)]


def build(force: bool = False) -> Path:
    """Compile the oracle (gcc, OpenMP, no FMA contraction)."""
    src = HERE / "pbte_oracle.c"
    if LIB.exists() and not force and LIB.stat().st_mtime >= src.stat().st_mtime:
        return LIB
    LIB.parent.mkdir(exist_ok=True)
    tmp = LIB.with_suffix(f".{os.getpid()}.tmp")
    subprocess.run(["gcc", "-O2", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off",
                    "-fno-fast-math", str(src), "-o", str(tmp), "-lm"], check=True)
    os.replace(tmp, LIB)
    return LIB


_lib = None


def lib():
    global _lib
    if _lib is None:
        _lib = ctypes.CDLL(str(build()))
        _lib.orc_sweep.restype = ctypes.c_int
        _lib.orc_residual.restype = ctypes.c_double
        _lib.orc_sum.restype = ctypes.c_double
        _lib.orc_order.restype = ctypes.c_int
    return _lib


def _p(a):
    if a.dtype == np.float64:
        return a.ctypes.data_as(_d)
    return a.ctypes.data_as(_i)


def reference_order(disc, allow_break: bool = False):
    """pybte's TRI_ORDER (``ordering.py:61-140``) for every direction."""
    cx, cy, _ = disc.vel.flat()
    m = disc.mesh
    nt, ndir = m.n_tris, cx.size
    order = np.full((ndir, nt), -1, dtype=np.int32)
    cycles = np.zeros(ndir, dtype=np.int32)
    nb = np.ascontiguousarray(m.tri_neighbour, dtype=np.int32)
    nx = np.ascontiguousarray(m.tri_normal[:, :, 0])
    ny = np.ascontiguousarray(m.tri_normal[:, :, 1])
    st = lib().orc_order(ndir, nt, _p(nb), _p(nx), _p(ny), _p(np.ascontiguousarray(cx)),
                         _p(np.ascontiguousarray(cy)), _p(order), _p(cycles), int(allow_break))
    if st != 0:
        raise RuntimeError("sweep graph has a cycle")
    return order, cycles


class Oracle:
    """The reference solver restated: state ``vdf`` (ndir, n_tris, nd) and the
    moments ``ts, qxs, qys`` (nd, n_tris), ``temp, qx, qy`` (n_tris,)."""

    def __init__(self, disc, nthreads: int | None = None, order=None):
        c = disc.case
        self.disc = disc
        m, it, bd = disc.mesh, disc.integrals, disc.bcdata
        self.nthreads = nthreads or (os.cpu_count() or 1)
        cx, cy, dw = disc.vel.flat()
        self.cxv, self.cyv, self.domega = (np.ascontiguousarray(v) for v in (cx, cy, dw))
        self.order, self.cycles = (order if order is not None else reference_order(disc))
        self.nt, self.nd, self.ndir = m.n_tris, disc.ndof, cx.size
        self.arr = dict(
            mass=np.ascontiguousarray(it.int_tri_tri), gx=np.ascontiguousarray(it.int_tri_tri_x),
            gy=np.ascontiguousarray(it.int_tri_tri_y), fcm=np.ascontiguousarray(it.int_tri_fc),
            ttfc=np.ascontiguousarray(it.int_tri_tri_fc),
            nx=np.ascontiguousarray(m.tri_normal[:, :, 0]), ny=np.ascontiguousarray(m.tri_normal[:, :, 1]),
            tri_faces=np.ascontiguousarray(m.tri_faces, dtype=np.int32),
            face_bc=np.ascontiguousarray(m.face_bc, dtype=np.int32),
            neighbour=np.ascontiguousarray(m.tri_neighbour, dtype=np.int32),
            periodic_tri=np.ascontiguousarray(bd.periodic_tri, dtype=np.int32),
            bc_type=np.ascontiguousarray(bd.bc_type, dtype=np.int32),
            bc_temp=np.ascontiguousarray(bd.bc_temp))
        self.flux_wall = np.zeros((m.n_faces, self.nd))
        self.pbuf = np.zeros((self.ndir, m.n_faces, self.nd))
        self.use_pbuf = False
        self.int_tri = np.ascontiguousarray(it.int_tri)
        self.fcm = self.arr["fcm"]
        self.face_tri = np.ascontiguousarray(m.face_tri, dtype=np.int32)
        self.face_lfc = np.ascontiguousarray(m.face_lfc, dtype=np.int32)
        a = self.arr
        self.ctx = OrcCtx(self.ndir, self.nt, self.nd, m.n_faces, bd.bc_type.size,
                          _p(self.order), _p(self.cxv), _p(self.cyv), _p(self.domega),
                          c.flow.cv, c.flow.vg, c.flow.tau_r, c.flow.tau_n, c.tau_c, PI,
                          _p(a["mass"]), _p(a["gx"]), _p(a["gy"]), _p(a["fcm"]), _p(a["ttfc"]),
                          _p(a["nx"]), _p(a["ny"]), _p(a["tri_faces"]), _p(a["face_bc"]),
                          _p(a["neighbour"]), _p(a["periodic_tri"]), _p(a["bc_type"]),
                          _p(a["bc_temp"]), _p(self.flux_wall))
        self.reset()
        self.sweep_count = 0

    def reset(self):
        self.vdf = np.zeros((self.ndir, self.nt, self.nd))
        self.ts = np.zeros((self.nd, self.nt))
        self.qxs = np.zeros((self.nd, self.nt))
        self.qys = np.zeros((self.nd, self.nt))
        self.temp = np.zeros(self.nt)
        self.qx = np.zeros(self.nt)
        self.qy = np.zeros(self.nt)
        self.flux_wall[:] = 0.0

    # -- kernels ----------------------------------------------------------
    def sweep(self):
        bad = lib().orc_sweep(ctypes.byref(self.ctx), _p(self.ts), _p(self.qxs), _p(self.qys),
                              _p(self.vdf), _p(self.pbuf), int(self.use_pbuf), self.nthreads)
        self.sweep_count += 1
        if bad:
            raise np.linalg.LinAlgError(f"{bad} singular element operators")

    def moments(self):
        lib().orc_moments(self.ndir, self.nt, self.nd, _p(self.vdf), _p(self.cxv), _p(self.cyv),
                          _p(self.domega), _p(self.int_tri), ctypes.c_double(self.disc.case.flow.cv),
                          _p(self.ts), _p(self.qxs), _p(self.qys), _p(self.temp), _p(self.qx), _p(self.qy))

    def wall_flux(self):
        if not self.disc.bcdata.has_nonthermalising:
            return
        lib().orc_wall_flux(self.ndir, self.nt, self.nd, self.disc.mesh.n_faces, _p(self.vdf),
                            _p(self.cxv), _p(self.cyv), _p(self.domega), _p(self.fcm),
                            _p(self.arr["nx"]), _p(self.arr["ny"]), _p(self.arr["face_bc"]),
                            _p(self.face_tri), _p(self.face_lfc), _p(self.arr["bc_type"]),
                            _p(self.flux_wall))

    def residual(self, t_old) -> float:
        return float(lib().orc_residual(_p(self.temp), _p(t_old), self.nt))

    @property
    def mass(self) -> float:
        return float(lib().orc_sum(_p(self.temp), self.nt))

    def true_residual(self) -> float:
        num = np.zeros(self.ndir)
        den = np.zeros(self.ndir)
        lib().orc_transport_residual(ctypes.byref(self.ctx), _p(self.ts), _p(self.qxs), _p(self.qys),
                                     _p(self.vdf), _p(self.pbuf), _p(num), _p(den), self.nthreads)
        d = float(den.sum())
        return float("nan") if d <= 0.0 else float(np.sqrt(num.sum() / d))

    # -- CIS: pybte/driver.py:149-215 --------------------------------------
    def step(self, acc=None):
        self.wall_flux()
        self.sweep()
        if acc is None:
            self.moments()
        else:
            acc.apply()

    def run_source(self, tol=None, tmax=None, gsis: bool = False):
        c = self.disc.case
        tol = c.iteration.tol if tol is None else tol
        tmax = c.iteration.tmax if tmax is None else tmax
        acc = GSIS(self) if gsis else None
        t_old = np.zeros(self.nt)
        res_hist, mass_hist = [], []
        step, converged = 0, False
        t0 = time.perf_counter()
        while True:
            step += 1
            self.step(acc)
            res = self.residual(t_old)
            t_old[:] = self.temp
            res_hist.append(res)
            mass_hist.append(self.mass)
            if res < tol:
                converged = True
                break
            if step >= tmax:
                break
        return dict(iterations=step, converged=converged, residuals=np.array(res_hist),
                    masses=np.array(mass_hist), wall=time.perf_counter() - t0)

    # -- GMRES: pybte/krylov.py -----------------------------------------------
    def run_krylov(self, tol=None, tmax=None, max_basis=None):
        c = self.disc.case
        tol = c.iteration.tol if tol is None else tol
        tmax = c.iteration.tmax if tmax is None else tmax
        if int(self.cycles.sum()):
            raise ValueError("Krylov acceleration does not apply: broken cycles")
        op = _FixedPoint(self)
        try:
            return _run_krylov(self, op, tol, tmax, c.scheme, max_basis)
        finally:
            self.use_pbuf = False


class _FixedPoint:
    """``pybte/krylov.py:64-136``: the state is the moments, the wall emission
    (if adiabatic walls) and the periodic partner DOFs."""

    def __init__(self, o: Oracle):
        self.o = o
        self.nmom = 3 * o.nd * o.nt
        self.wall = bool(o.disc.bcdata.has_nonthermalising)
        self.nwall = o.flux_wall.size if self.wall else 0
        self.per = bool(o.disc.bcdata.has_periodic)
        self.pfaces = (np.flatnonzero(o.arr["periodic_tri"] >= 0) if self.per else np.zeros(0, dtype=np.int64))
        self.ptri = o.arr["periodic_tri"][self.pfaces]
        self.nper = o.ndir * self.pfaces.size * o.nd if self.per else 0
        self.n = self.nmom + self.nwall + self.nper
        o.use_pbuf = self.per

    def scatter(self, u):
        o = self.o
        k = o.nd * o.nt
        np.copyto(o.ts, u[:k].reshape(o.ts.shape))
        np.copyto(o.qxs, u[k:2 * k].reshape(o.qxs.shape))
        np.copyto(o.qys, u[2 * k:3 * k].reshape(o.qys.shape))
        if self.wall:
            np.copyto(o.flux_wall, u[self.nmom:self.nmom + self.nwall].reshape(o.flux_wall.shape))
        if self.per:
            o.pbuf[:, self.pfaces, :] = u[self.nmom + self.nwall:].reshape(o.ndir, self.pfaces.size, o.nd)

    def gather(self):
        o = self.o
        u = np.empty(self.n)
        k = o.nd * o.nt
        u[:k] = o.ts.reshape(-1)
        u[k:2 * k] = o.qxs.reshape(-1)
        u[2 * k:3 * k] = o.qys.reshape(-1)
        if self.wall:
            u[self.nmom:self.nmom + self.nwall] = o.flux_wall.reshape(-1)
        if self.per:
            u[self.nmom + self.nwall:] = o.vdf[:, self.ptri, :].reshape(-1)
        return u

    def apply(self, u):
        o = self.o
        self.scatter(u)
        o.sweep()
        o.moments()
        o.wall_flux()
        return self.gather()

    def state(self):
        self.o.moments()
        self.o.wall_flux()
        return self.gather()


def _back_substitute(r, y):
    out = np.array(y, dtype=float)
    for i in range(out.size - 1, -1, -1):
        s = out[i] - r[i, i + 1:] @ out[i + 1:]
        out[i] = s / r[i, i] if r[i, i] != 0.0 else 0.0
    return out


def gmres_full(matvec, b, x0=None, tol_abs=0.0, maxiter=None, max_basis=None, callback=None):
    """``pybte/krylov.py:150-246``: classical Gram-Schmidt applied twice,
    Givens rotations, restart at ``max_basis``."""
    n = b.shape[0]
    x = np.zeros(n) if x0 is None else np.array(x0, dtype=float)
    maxiter = int(n if maxiter is None else maxiter)
    m_cap = maxiter if max_basis is None else max(1, min(int(max_basis), maxiter))
    nmv = 0
    converged = halted = False
    while nmv < maxiter and not converged and not halted:
        if np.any(x):
            r = b - matvec(x)
            nmv += 1
            if callback is not None and callback(float(np.sqrt(r @ r))):
                halted = True
                break
        else:
            r = b.copy()
        beta = float(np.sqrt(r @ r))
        if beta <= tol_abs:
            converged = True
            break
        m = min(m_cap, maxiter - nmv)
        if m <= 0:
            break
        q = np.empty((min(m, 64), n))
        q[0] = r / beta
        cols, cs, sn, gam = [], [], [], [beta]
        for j in range(m):
            w = matvec(q[j])
            nmv += 1
            qj = q[:j + 1]
            c1 = qj @ w
            w -= qj.T @ c1
            c2 = qj @ w
            w -= qj.T @ c2
            col = np.empty(j + 2)
            col[:j + 1] = c1 + c2
            hn = float(np.sqrt(w @ w))
            col[j + 1] = hn
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
                    grown = np.empty((min(m, max(2 * q.shape[0], j + 2)), n))
                    grown[:j + 1] = q[:j + 1]
                    q = grown
                q[j + 1] = w / hn
        k = len(cols)
        if k:
            rmat = np.zeros((k, k))
            for j, col in enumerate(cols):
                rmat[:j + 1, j] = col
            x += q[:k].T @ _back_substitute(rmat, np.asarray(gam[:k]))
    return x, converged, nmv


def _run_krylov(o: Oracle, op: _FixedPoint, tol, tmax, scheme, max_basis):
    """``pybte/krylov.py:285-363``; ``iterations`` counts sweeps."""
    residuals, masses = [], []

    def sweep(u):
        out = op.apply(u)
        masses.append(o.mass)
        residuals.append(np.nan)
        return out

    g = sweep(np.zeros(op.n))
    gnorm = float(np.sqrt(g @ g))
    scale = gnorm or 1.0
    residuals[-1] = 1.0
    x = np.zeros(op.n)

    def matvec(v):
        return v - (sweep(v) - g)

    enough = max(tol * 1.0e-2, 1.0e-14) * scale
    target = max(tol * scheme.krylov_tol_factor, 1.0e-14) * scale
    if max_basis is None:
        per = max(1.0, 8.0 * float(op.n))
        max_basis = int(max(32, min(int(tmax), int(scheme.krylov_max_bytes / per))))
    reached = -1

    def on_residual(res):
        nonlocal reached
        residuals[-1] = res / scale
        n = len(residuals)
        if reached < 0 and res <= enough:
            reached = n
        return reached >= 0 and n - reached > max(64, reached // 4)

    converged = False
    final = float("nan")
    for _ in range(scheme.krylov_max_rounds):
        budget = tmax - len(residuals) - 1
        if budget <= 0:
            break
        reached = -1
        x, _, _ = gmres_full(matvec, g, x0=x, tol_abs=target, maxiter=budget,
                             max_basis=max_basis, callback=on_residual)
        sweep(x)
        final = o.true_residual()
        residuals[-1] = final
        converged = bool(final < tol) if np.isfinite(final) else gnorm == 0.0
        if converged or len(residuals) >= tmax:
            break
        target = max(target * 1.0e-3, 1.0e-14 * scale)
    return dict(iterations=len(residuals), converged=converged, transport_residual=final,
                residuals=np.array(residuals), masses=np.array(masses), krylov_size=op.n,
                basis=max_basis)


# ---------------------------------------------------------------------------
# GSIS: pybte/acceleration/*.py
# ---------------------------------------------------------------------------
def _mirror_perm(nf):
    base = np.arange(nf)[::-1]
    return np.concatenate([base + b * nf for b in range(3)])


class GSIS:
    """``pybte/acceleration/__init__.py:34-115`` with the shipped defaults
    (defect repair off)."""

    def __init__(self, o: Oracle):
        from scipy.sparse import coo_matrix
        from scipy.sparse.linalg import splu

        self.o = o
        disc = o.disc
        c, m, it = disc.case, disc.mesh, disc.integrals
        nd, nf = disc.ndof, c.ndof_fc
        self.nd, self.nf = nd, nf
        variant = c.scheme.acc_variant
        self.variant = variant
        st = np.asarray(c.scheme.stabilisation, dtype=float).copy()
        if c.scheme.scale_by_hmin:
            st[1] /= m.hmin
            st[2] /= m.hmin
        bc_type = disc.bcdata.bc_type
        tau_r, tau_c, cv = c.flow.tau_r, c.tau_c, c.flow.cv
        scale = tau_r if variant == "B" else 1.0
        n_tris = m.n_tris

        # build_local_operators: assembly.py:44-125
        aa = it.int_tri_tri_x
        bb = it.int_tri_tri_y
        cc = np.transpose(aa, (0, 2, 1)).copy()
        dd = np.transpose(bb, (0, 2, 1)).copy()
        pp = it.int_tri_fc.sum(axis=1)
        oo = np.transpose(it.int_tri_tri, (2, 0, 1)).copy()
        A = np.zeros((n_tris, 7 * nd, 7 * nd))

        def blk(r, cl):
            return A[:, r * nd:(r + 1) * nd, cl * nd:(cl + 1) * nd]
        blk(0, 0)[:] = st[0] * pp
        blk(0, 1)[:] = cc
        blk(0, 2)[:] = dd
        blk(1, 0)[:] = -aa * cv / 3.0 * scale
        blk(1, 1)[:] = (oo + st[1] * pp) if variant == "B" else (st[1] * pp + oo / tau_r)
        blk(1, 3)[:] = -4.0 / 3.0 * cc
        blk(1, 4)[:] = -dd
        blk(1, 5)[:] = -dd
        blk(1, 6)[:] = 2.0 / 3.0 * cc
        blk(2, 0)[:] = -bb * cv / 3.0 * scale
        blk(2, 2)[:] = (oo + st[2] * pp) if variant == "B" else (st[2] * pp + oo / tau_r)
        blk(2, 3)[:] = 2.0 / 3.0 * dd
        blk(2, 4)[:] = -cc
        blk(2, 5)[:] = -cc
        blk(2, 6)[:] = -4.0 / 3.0 * dd
        tc5 = tau_c * scale / 5.0
        blk(3, 1)[:] = aa * tc5
        blk(3, 3)[:] = oo
        blk(4, 1)[:] = bb * tc5
        blk(4, 4)[:] = oo
        blk(5, 2)[:] = aa * tc5
        blk(5, 5)[:] = oo
        blk(6, 2)[:] = bb * tc5
        blk(6, 6)[:] = oo
        self.inv_aa_sol = np.linalg.inv(A)
        ww = np.transpose(it.int_tri_fc_fc, (2, 3, 0, 1)).copy()
        nx = m.tri_normal[:, :, 0]
        ny = m.tri_normal[:, :, 1]
        T = np.zeros((n_tris, 3, 7 * nd, 3 * nf))

        def tblk(r, cl):
            return T[:, :, r * nd:(r + 1) * nd, cl * nf:(cl + 1) * nf]
        nxe = nx[:, :, None, None]
        nye = ny[:, :, None, None]
        tblk(0, 0)[:] = st[0] * ww
        tblk(1, 0)[:] = -nxe * ww * cv / 3.0 * scale
        tblk(1, 1)[:] = st[1] * ww
        tblk(2, 0)[:] = -nye * ww * cv / 3.0 * scale
        tblk(2, 2)[:] = st[2] * ww
        tblk(3, 1)[:] = nxe * ww * tc5
        tblk(4, 1)[:] = nye * ww * tc5
        tblk(5, 2)[:] = nxe * ww * tc5
        tblk(6, 2)[:] = nye * ww * tc5
        self.aa_trace = np.einsum("ipq,ilqr->ilpr", self.inv_aa_sol, T, optimize=True)

        # build_ba_sol: assembly.py:128-184
        B = np.zeros((n_tris, 3, 3 * nf, 7 * nd))
        bb2 = np.transpose(it.int_tri_fc_fc, (2, 3, 1, 0)).copy()
        nxb = nx[:, :, None, None]
        nyb = ny[:, :, None, None]

        def bblk(r, cl):
            return B[:, :, r * nf:(r + 1) * nf, cl * nd:(cl + 1) * nd]
        face_bc = m.face_bc[m.tri_faces]
        code = np.where(face_bc >= 0, bc_type[np.clip(face_bc, 0, None)], 0)
        interior = face_bc < 0
        periodic = (~interior) & (code == 3)
        wall_th = (~interior) & (code == 1)
        std = (interior | periodic)[:, :, None, None]
        bblk(0, 0)[:] = np.where(std, 0.5 * bb2, 0.0)
        bblk(0, 1)[:] = np.where(std, nxb / 2.0 / st[0] * bb2, 0.0)
        bblk(0, 2)[:] = np.where(std, nyb / 2.0 / st[0] * bb2, 0.0)
        bblk(1, 1)[:] = np.where(std, 0.5 * bb2, 0.0)
        bblk(1, 3)[:] = np.where(std, -2.0 * nxb / 3.0 / st[1] * bb2, 0.0)
        bblk(1, 4)[:] = np.where(std, -nyb / 2.0 / st[1] * bb2, 0.0)
        bblk(1, 5)[:] = np.where(std, -nyb / 2.0 / st[1] * bb2, 0.0)
        bblk(1, 6)[:] = np.where(std, nxb / 3.0 / st[1] * bb2, 0.0)
        bblk(2, 2)[:] = np.where(std, 0.5 * bb2, 0.0)
        bblk(2, 3)[:] = np.where(std, nyb / 3.0 / st[2] * bb2, 0.0)
        bblk(2, 4)[:] = np.where(std, -nxb / 2.0 / st[2] * bb2, 0.0)
        bblk(2, 5)[:] = np.where(std, -nxb / 2.0 / st[2] * bb2, 0.0)
        bblk(2, 6)[:] = np.where(std, -2.0 * nyb / 3.0 / st[2] * bb2, 0.0)
        if variant == "A":
            w = wall_th[:, :, None, None]
            bblk(1, 1)[:] = np.where(w, bb2, bblk(1, 1))
            bblk(1, 3)[:] = np.where(w, -4.0 * nxb / 3.0 / st[1] * bb2, bblk(1, 3))
            bblk(1, 4)[:] = np.where(w, -nyb / st[1] * bb2, bblk(1, 4))
            bblk(1, 5)[:] = np.where(w, -nyb / st[1] * bb2, bblk(1, 5))
            bblk(1, 6)[:] = np.where(w, 2.0 * nxb / 3.0 / st[1] * bb2, bblk(1, 6))
            bblk(2, 2)[:] = np.where(w, bb2, bblk(2, 2))
            bblk(2, 3)[:] = np.where(w, 2.0 * nyb / 3.0 / st[2] * bb2, bblk(2, 3))
            bblk(2, 4)[:] = np.where(w, -nxb / st[2] * bb2, bblk(2, 4))
            bblk(2, 5)[:] = np.where(w, -nxb / st[2] * bb2, bblk(2, 5))
            bblk(2, 6)[:] = np.where(w, -4.0 * nyb / 3.0 / st[2] * bb2, bblk(2, 6))
        self.ba_sol = B

        # assemble_global_matrix: assembly.py:200-269
        nf3 = 3 * nf
        n_faces = m.n_faces
        perm = _mirror_perm(nf)
        flipv = disc.bcdata.periodic_flip
        drop = 1e-30 if variant == "A" else 0.0
        rows, cols, vals = [], [], []
        rr, ccg = np.meshgrid(np.arange(nf3), np.arange(nf3), indexing="ij")
        aa_tmp = np.zeros((nf3, nf3))
        for f in range(n_faces):
            aaf = it.int_fc_fc[:, :, f]
            aa_tmp[:] = 0.0
            for k in range(3):
                aa_tmp[k * nf:(k + 1) * nf, k * nf:(k + 1) * nf] = aaf
            blocks = {f: aa_tmp.copy()}
            bc = int(m.face_bc[f])
            if bc < 0:
                t1, t2 = m.face_tri[f]
                l1, l2 = m.face_lfc[f]
                pairs = [(int(t1), int(l1), False), (int(t2), int(l2), False)]
            elif bc_type[bc] == 3:
                t1, l1 = m.adjacent(f)
                t2, l2 = m.adjacent(int(m.face_pair[f]))
                pairs = [(t1, l1, False), (t2, l2, bool(flipv[f]))]
            else:
                t1, l1 = m.adjacent(f)
                pairs = [(t1, l1, False)]
            for tri, lfc, mirror in pairs:
                for il in range(3):
                    gface = int(m.tri_faces[tri, il])
                    dmat = self.ba_sol[tri, lfc] @ self.aa_trace[tri, il]
                    if mirror:
                        dmat = dmat[perm]
                    if gface in blocks:
                        blocks[gface] -= dmat
                    else:
                        blocks[gface] = -dmat
            for gface, bl in blocks.items():
                keep = np.abs(bl) > drop
                if not keep.any():
                    continue
                rows.append(f * nf3 + rr[keep])
                cols.append(gface * nf3 + ccg[keep])
                vals.append(bl[keep])
        n = n_faces * nf3
        K = coo_matrix((np.concatenate(vals), (np.concatenate(rows), np.concatenate(cols))),
                       shape=(n, n)).tocsr()
        K.sort_indices()
        self.K = K
        self.lu = splu(K.tocsc())
        self.perm = perm

        # GlobalSolver bookkeeping: global_solve.py:68-117
        p1_tri = np.full(n_faces, -1, dtype=np.int64)
        p1_lfc = np.full(n_faces, -1, dtype=np.int64)
        p2_tri = np.full(n_faces, -1, dtype=np.int64)
        p2_lfc = np.full(n_faces, -1, dtype=np.int64)
        for f in range(n_faces):
            bc = int(m.face_bc[f])
            if bc < 0:
                p1_tri[f], p2_tri[f] = m.face_tri[f]
                p1_lfc[f], p2_lfc[f] = m.face_lfc[f]
            elif bc_type[bc] == 3:
                p1_tri[f], p1_lfc[f] = m.adjacent(f)
                p2_tri[f], p2_lfc[f] = m.adjacent(int(m.face_pair[f]))
            else:
                p1_tri[f], p1_lfc[f] = m.adjacent(f)
        self.p1_tri, self.p1_lfc, self.p2_tri, self.p2_lfc = p1_tri, p1_lfc, p2_tri, p2_lfc
        self.has_p2 = p2_tri >= 0
        codes = np.where(m.face_bc >= 0, bc_type[np.clip(m.face_bc, 0, None)], 0)
        self.wall_th = np.flatnonzero((m.face_bc >= 0) & (codes == 1))
        self.wall_ad = np.flatnonzero((m.face_bc >= 0) & (codes == 2))
        self.wall_all = np.concatenate([self.wall_th, self.wall_ad])
        self.wall_tri = np.ascontiguousarray(p1_tri[self.wall_all], dtype=np.int32)
        self.wall_lfc = np.ascontiguousarray(p1_lfc[self.wall_all], dtype=np.int32)
        self.n_th = self.wall_th.size
        self.wall_nx = m.tri_normal[self.wall_tri, self.wall_lfc, 0]
        self.wall_ny = m.tri_normal[self.wall_tri, self.wall_lfc, 1]
        self.flip = flipv
        self.tri_fc_fc = np.ascontiguousarray(it.int_tri_fc_fc)
        self.gx_t = np.ascontiguousarray(it.int_tri_tri_x)
        self.gy_t = np.ascontiguousarray(it.int_tri_tri_y)
        self.tc5 = tc5
        self.use_hmin = variant == "A"
        self.work = np.zeros((n_tris, 7 * nd))
        self.solve_count = 0

    def apply(self):
        """``Acceleration.apply``: hot source, trace rhs + solve, local recovery,
        damped correction of vdf and the moments."""
        o, c = self.o, self.o.disc.case
        nd, nf = self.nd, self.nf
        m = o.disc.mesh
        self.work[:] = 0.0
        lib().orc_hot_kernel(o.ndir, o.nt, nd, _p(o.vdf), _p(self.gx_t), _p(self.gy_t), _p(o.cxv),
                             _p(o.cyv), _p(o.domega), ctypes.c_double(self.tc5), _p(self.work))
        aa_src = np.ascontiguousarray(np.einsum("ipq,iq->pi", self.inv_aa_sol, self.work, optimize=True))
        # GlobalSolver.rhs: global_solve.py:131-187
        nf3 = 3 * nf
        ffa = np.zeros((nf3, m.n_faces))
        ffa[:] = np.einsum("fpq,qf->pf", self.ba_sol[self.p1_tri, self.p1_lfc],
                           aa_src[:, self.p1_tri], optimize=True)
        sel = self.has_p2
        if sel.any():
            c2 = np.einsum("fpq,qf->pf", self.ba_sol[self.p2_tri[sel], self.p2_lfc[sel]],
                           aa_src[:, self.p2_tri[sel]], optimize=True)
            fl = self.flip[sel]
            if fl.any():
                c2[:, fl] = c2[self.perm][:, fl]
            ffa[:, sel] += c2
        if self.wall_all.size:
            mom = np.zeros((self.wall_all.size, nf3))
            lib().orc_wall_trace(o.ndir, o.nt, nd, nf, _p(o.vdf), _p(self.tri_fc_fc), _p(o.cxv),
                                 _p(o.cyv), _p(o.domega), int(self.wall_all.size),
                                 _p(self.wall_tri), _p(self.wall_lfc), _p(mom))
            th = self.wall_all[:self.n_th]
            ad = self.wall_all[self.n_th:]
            cv = c.flow.cv
            if th.size:
                ffa[0:nf, th] = mom[:self.n_th, 0:nf].T / cv
                if self.variant == "B":
                    ffa[nf:2 * nf, th] = mom[:self.n_th, nf:2 * nf].T
                    ffa[2 * nf:3 * nf, th] = mom[:self.n_th, 2 * nf:3 * nf].T
            if ad.size:
                ffa[0:nf, ad] = mom[self.n_th:, 0:nf].T / cv
                qxb = mom[self.n_th:, nf:2 * nf].T
                qyb = mom[self.n_th:, 2 * nf:3 * nf].T
                nx = self.wall_nx[self.n_th:]
                ny = self.wall_ny[self.n_th:]
                ffa[nf:2 * nf, ad] = qxb * (ny * ny) - qyb * (nx * ny)
                ffa[2 * nf:3 * nf, ad] = -qxb * (nx * ny) + qyb * (nx * nx)
        x = self.lu.solve(ffa.ravel(order="F"))
        self.solve_count += 1
        u_trace = x.reshape(nf3, m.n_faces, order="F")
        # local_solve.py:16-26
        uq = aa_src.copy()
        traces = u_trace[:, m.tri_faces]
        uq += np.einsum("ilpr,ril->pi", self.aa_trace, traces, optimize=True)
        self.uq = uq
        self.aa_src = aa_src
        self.ffa = ffa
        self.u_trace = u_trace
        # correction.py:78-98
        lib().orc_correct(o.ndir, o.nt, nd, _p(o.vdf), _p(np.ascontiguousarray(uq)), _p(o.cxv),
                          _p(o.cyv), _p(o.domega), _p(o.int_tri),
                          _p(np.ascontiguousarray(m.tri_hmin)), ctypes.c_double(c.flow.cv),
                          ctypes.c_double(c.flow.vg), ctypes.c_double(c.flow.tau_r),
                          ctypes.c_double(c.flow.tau_n), ctypes.c_double(c.tau_c),
                          ctypes.c_double(c.flow.tau_thr), ctypes.c_double(PI),
                          int(self.use_hmin), _p(o.ts), _p(o.qxs), _p(o.qys), _p(o.temp),
                          _p(o.qx), _p(o.qy))
