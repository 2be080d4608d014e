"""GPU transport sweep behind pybte's ``SweepContext`` interface.

``SweepContext`` here has the reference's surface (``pybte/sweep.py:37-197``):
``sweep(mom, vdf)`` updates ``vdf`` in place and increments ``sweep_count``;
``true_residual(mom, vdf)`` returns the weighted transport residual; the
attributes ``cxv, cyv, domega, mode, kernel, sweep_count, use_pbuf, pbuf,
flux_wall, operator_bytes()`` are present.  ``vdf`` and the moments may be
CUDA tensors (kept resident) or host numpy arrays (copied in and out, so a
caller written for pybte works unchanged).

The work runs in ``libpbte_gb300.so`` through its C ABI; torch supplies the
device buffers and the stream.  There is no CPU fallback.
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass

import numpy as np
import torch

from . import _lib
from .device import device_lock, empty_graveyard
from .discretisation import Discretisation

__all__ = ["SweepContext", "Moments", "device_ptr", "SweepCycleError", "HostReadable"]


class SweepCycleError(RuntimeError):
    """A direction's element dependency graph contains a cycle
    (``pybte/ordering.py:35``); raised where pybte's default
    ``on_cycle='raise'`` raises it."""


class HostReadable(torch.Tensor):
    """A device tensor that numpy reads by copying it to the host, so that
    ``np.asarray(solver.vdf)`` works as it does on pybte's host array (the
    reference task's verifier saves the distribution that way)."""

    def __array__(self, dtype=None, copy=None):
        a = torch.Tensor.cpu(self).detach().numpy()
        return a if dtype is None else a.astype(dtype, copy=False)


def _create_status(rc: int, what: str) -> None:
    """pybte's exceptions for the context's failures: singular element
    operators raise LinAlgError (``sweep.py:122-128``), a cyclic direction
    SweepCycleError (``ordering.py:169``)."""
    if rc == -6:
        raise np.linalg.LinAlgError("element operators are singular; check TAU_C and the mesh")
    if rc == -3:
        raise SweepCycleError("a direction has a cyclic element dependency; the mesh is not sweepable for it")
    _lib.check(rc, what)

# contexts whose destruction waits for a moment outside graph captures
_deferred: list = []


def _destroy_deferred() -> None:
    """Destroy the contexts queued by SweepContext.__del__ (caller holds
    device_lock)."""
    while _deferred:
        h = _deferred.pop()
        try:
            _lib.lib().pbte_ctx_destroy(h)
        except Exception:
            pass


def device_ptr(t) -> int:
    if t is None:
        return 0
    return t.data_ptr()


def _stream(stream=None) -> int:
    s = stream if stream is not None else torch.cuda.current_stream()
    return s.cuda_stream


@dataclass
class Moments:
    """Per-DOF and per-element macroscopic fields (``pybte/moments.py:29-47``)
    as device tensors: ``ts, qxs, qys`` (ndof, n_tris); ``temp, qx, qy`` (n_tris,)."""
    ts: torch.Tensor
    qxs: torch.Tensor
    qys: torch.Tensor
    temp: torch.Tensor
    qx: torch.Tensor
    qy: torch.Tensor

    @property
    def mass(self) -> float:
        return float(self.temp.sum().item())

    @classmethod
    def zeros(cls, ndof: int, n_tris: int, device="cuda") -> "Moments":
        z = lambda *s: torch.zeros(s, dtype=torch.float64, device=device)  # noqa: E731
        return cls(z(ndof, n_tris), z(ndof, n_tris), z(ndof, n_tris), z(n_tris), z(n_tris), z(n_tris))

    def host(self) -> dict:
        return {k: getattr(self, k).detach().cpu().numpy() for k in
                ("ts", "qxs", "qys", "temp", "qx", "qy")}


def case_desc(disc: Discretisation):
    """The ``pbte_case_desc`` of a case and the host arrays it points into
    (keep them alive while the descriptor is used)."""
    c = disc.case
    it, m, bd = disc.integrals, disc.mesh, disc.bcdata
    cx, cy, dw = disc.vel.flat()
    a = dict(
        cxv=np.ascontiguousarray(cx), cyv=np.ascontiguousarray(cy), domega=np.ascontiguousarray(dw),
        ref_mass=np.ascontiguousarray(it.ref_mass), ref_dx=np.ascontiguousarray(it.ref_dx),
        ref_dy=np.ascontiguousarray(it.ref_dy), ref_edge=np.ascontiguousarray(it.ref_edge),
        edge_dofs=np.ascontiguousarray(disc.edge_dofs, dtype=np.int32),
        area2=np.ascontiguousarray(it.area2), dxi=np.ascontiguousarray(it.dxi),
        deta=np.ascontiguousarray(it.deta), edge_scale=np.ascontiguousarray(it.edge_scale),
        nx=np.ascontiguousarray(m.tri_normal[:, :, 0]), ny=np.ascontiguousarray(m.tri_normal[:, :, 1]),
        tri_faces=np.ascontiguousarray(m.tri_faces, dtype=np.int32),
        upwind_tri=np.ascontiguousarray(disc.upwind_tri, dtype=np.int32),
        edge_map=np.ascontiguousarray(disc.edge_map, dtype=np.int32),
        face_bc=np.ascontiguousarray(m.face_bc, dtype=np.int32),
        face_tri=np.ascontiguousarray(m.face_tri, dtype=np.int32),
        face_lfc=np.ascontiguousarray(m.face_lfc, dtype=np.int32),
        bc_type=np.ascontiguousarray(bd.bc_type, dtype=np.int32),
        bc_temp=np.ascontiguousarray(bd.bc_temp), int_tri=np.ascontiguousarray(it.int_tri))

    def P(x):
        return x.ctypes.data_as(ctypes.POINTER(ctypes.c_int32 if x.dtype == np.int32 else ctypes.c_double))

    desc = _lib.CaseDesc(m.n_tris, m.n_faces, disc.ndof, c.ndof_fc, cx.size,
                         int(bd.bc_type.size), c.flow.cv, c.flow.vg, c.flow.tau_r, c.flow.tau_n,
                         c.tau_c, *(P(a[k]) for k in (
                             "cxv", "cyv", "domega", "ref_mass", "ref_dx", "ref_dy", "ref_edge",
                             "edge_dofs", "area2", "dxi", "deta", "edge_scale", "nx", "ny",
                             "tri_faces", "upwind_tri", "edge_map", "face_bc", "face_tri",
                             "face_lfc", "bc_type", "bc_temp", "int_tri")))
    return desc, a


def direction_classes(disc: Discretisation) -> np.ndarray:
    """Each ordinate's direction class, as the context schedules them
    (``pbte_direction_classes``; host only)."""
    desc, keep = case_desc(disc)
    out = np.zeros(disc.vel.flat()[0].size, dtype=np.int32)
    n = ctypes.c_int32()
    _lib.check(_lib.lib().pbte_direction_classes(ctypes.byref(desc), out.ctypes.data, ctypes.byref(n)),
               "pbte_direction_classes")
    del keep
    return out


def direction_levels(disc: Discretisation, d: int) -> np.ndarray:
    """The wavefront level of every element for ordinate ``d``, as the
    context schedules it (``pbte_direction_levels``; host only)."""
    desc, keep = case_desc(disc)
    out = np.zeros(disc.mesh.n_tris, dtype=np.int32)
    n = ctypes.c_int32()
    _create_status(_lib.lib().pbte_direction_levels(ctypes.byref(desc), int(d), out.ctypes.data, ctypes.byref(n)),
                   "pbte_direction_levels")
    del keep
    return out


class SweepContext:
    """The compact operators on the device plus the sweep schedule."""

    def __init__(self, disc: Discretisation, precompute: bool | None = None,
                 device: str = "cuda"):
        if not torch.cuda.is_available():
            raise RuntimeError("the GPU sweep needs a CUDA device; there is no CPU fallback")
        self.disc = disc
        c = disc.case
        it, m, bd = disc.integrals, disc.mesh, disc.bcdata
        self.device = torch.device(device)
        cx, cy, dw = disc.vel.flat()
        self.cxv, self.cyv, self.domega = (np.ascontiguousarray(v) for v in (cx, cy, dw))
        self.ndir, self.n_tris, self.ndof, self.n_faces = cx.size, m.n_tris, disc.ndof, m.n_faces
        self.cv, self.vg = c.flow.cv, c.flow.vg
        self.tau_r, self.tau_n, self.tau_c = c.flow.tau_r, c.flow.tau_n, c.tau_c
        self.kernel = "cuda"
        mode = c.performance.sweep_mode
        if precompute is None:
            if mode == "auto":
                # stored FP64 factors serve every FP64 sweep (the mixed path's
                # defect evaluations too); FP32 sweeps always factor in registers
                precompute = (c.performance.precompute_inverse
                              and self.operator_bytes(self.n_tris, self.ndof) <= c.performance.max_operator_bytes)
            else:
                precompute = mode == "precomputed"
        self.mode = "precomputed" if precompute else "onthefly"
        self.sweep_count = 0
        self.use_pbuf = False

        desc, self._host = case_desc(disc)
        handle = ctypes.c_void_p()
        with device_lock, torch.cuda.device(self.device):
            empty_graveyard()
            _destroy_deferred()
            _create_status(_lib.lib().pbte_ctx_create(ctypes.byref(desc), int(precompute),
                                                      ctypes.byref(handle)), "pbte_ctx_create")
        self._ctx = handle
        nlev, ncls, nbytes = ctypes.c_int64(), ctypes.c_int64(), ctypes.c_int64()
        _lib.check(_lib.lib().pbte_ctx_info(self._ctx, ctypes.byref(nlev), ctypes.byref(ncls),
                                            ctypes.byref(nbytes)), "pbte_ctx_info")
        self.n_levels_max, self.n_classes, self.device_bytes = nlev.value, ncls.value, nbytes.value
        f64 = dict(dtype=torch.float64, device=self.device)
        self.flux_wall = torch.zeros((self.n_faces, self.ndof), **f64)
        self.pbuf = torch.zeros((self.ndir if bd.has_periodic else 1,
                                 self.n_faces if bd.has_periodic else 1, self.ndof), **f64)
        self._num = torch.zeros(self.ndir, **f64)
        self._den = torch.zeros(self.ndir, **f64)
        self.lu = None   # the factors live inside the library in precomputed mode
        # stored FP32 factors for the FP32 sweeps, on request (same bits as
        # factoring in registers; measured no faster at P2, where the ring
        # sweep is bound by its level chain)
        self.fp32_factors = False
        if (c.performance.fp32_factors and self.ndof <= 10 and not bd.has_periodic
                and self.cxv.size * self.n_tris * self.ndof * self.ndof * 2.0 <= c.performance.max_operator_bytes):
            self.factorise_f32()

    def __del__(self):
        h = getattr(self, "_ctx", None)
        if h is not None and h.value:
            # destruction frees device memory (a device-wide synchronisation):
            # not while this thread captures a graph or another thread holds
            # the device lock; then it waits for the next context creation
            _deferred.append(ctypes.c_void_p(h.value))
            self._ctx = ctypes.c_void_p()
            try:
                capturing = torch.cuda.is_current_stream_capturing()
            except Exception:
                capturing = True
            if not capturing and device_lock.acquire(blocking=False):
                try:
                    _destroy_deferred()
                finally:
                    device_lock.release()

    @property
    def handle(self) -> ctypes.c_void_p:
        return self._ctx

    def set_variant(self, variant: int) -> None:
        """Sweep kernel: 0 automatic, 1 level-serial, 2 ring-pipelined only."""
        _lib.check(_lib.lib().pbte_set_sweep_variant(self._ctx, int(variant)), "pbte_set_sweep_variant")

    def set_groups(self, groups: int, width: int = 0) -> None:
        """Ring sweep block shape: pipeline depth (thread groups, 0: default)
        and threads per group (0: 64, or 64 or 128)."""
        _lib.check(_lib.lib().pbte_set_ring_groups(self._ctx, int(groups)), "pbte_set_ring_groups")
        _lib.check(_lib.lib().pbte_set_ring_width(self._ctx, int(width)), "pbte_set_ring_width")

    def factorise_f32(self, stream=None) -> None:
        """Store FP32 element factors (one set per distinct in-plane velocity)
        for the FP32 sweeps: same bits, no per-sweep assembly and
        factorisation (``pbte_factorise_f32``)."""
        _lib.check(_lib.lib().pbte_factorise_f32(self._ctx, _stream(stream)), "pbte_factorise_f32")
        nlev, ncls, nbytes = ctypes.c_int64(), ctypes.c_int64(), ctypes.c_int64()
        _lib.check(_lib.lib().pbte_ctx_info(self._ctx, ctypes.byref(nlev), ctypes.byref(ncls),
                                            ctypes.byref(nbytes)), "pbte_ctx_info")
        self.device_bytes = nbytes.value
        self.fp32_factors = True

    def singular_count(self, reset: bool = False) -> int:
        """Zero pivots met by the element factorisations so far (setup and
        every sweep that factors on the fly); synchronises the device."""
        v = ctypes.c_int64()
        _lib.check(_lib.lib().pbte_singular_count(self._ctx, ctypes.byref(v), int(reset)), "pbte_singular_count")
        return int(v.value)

    def schedule(self) -> dict:
        w, r, u = ctypes.c_int64(), ctypes.c_int64(), ctypes.c_int64()
        _lib.check(_lib.lib().pbte_ctx_schedule(self._ctx, ctypes.byref(w), ctypes.byref(r), ctypes.byref(u)),
                   "pbte_ctx_schedule")
        return {"ring_W": w.value, "ring_R": r.value, "unique_dirs": u.value,
                "levels": self.n_levels_max, "classes": self.n_classes}

    def operator_bytes(self, n_tris: int, ndof: int) -> float:
        """Bytes of stored FP64 factors (``pybte/sweep.py:113-114``)."""
        return float(self.cxv.size) * n_tris * ndof * ndof * 8.0

    # -- host/device plumbing for numpy callers ----------------------------
    def _dev(self, x, dtype=torch.float64):
        if isinstance(x, torch.Tensor):
            if x.device.type != "cuda" or x.dtype != dtype or not x.is_contiguous():
                raise ValueError("device arrays must be contiguous CUDA tensors of the right dtype")
            return x, False
        return torch.from_numpy(np.ascontiguousarray(x, dtype=np.float64)).to(self.device), True

    # -- the reference interface --------------------------------------------
    def sweep(self, mom, vdf, stream=None) -> None:
        """One transport sweep, in place on ``vdf`` (ndir, n_tris, ndof)."""
        ts, _ = self._dev(mom.ts)
        qxs, _ = self._dev(mom.qxs)
        qys, _ = self._dev(mom.qys)
        v, copied = self._dev(vdf)
        fw = self.flux_wall if isinstance(self.flux_wall, torch.Tensor) else self._dev(self.flux_wall)[0]
        _lib.check(_lib.lib().pbte_sweep(self._ctx, ts.data_ptr(), qxs.data_ptr(), qys.data_ptr(),
                                         v.data_ptr(), fw.data_ptr(), self.pbuf.data_ptr(),
                                         int(self.use_pbuf), _stream(stream)), "pbte_sweep")
        if copied:
            np.copyto(vdf, v.cpu().numpy())
        self.sweep_count += 1

    def true_residual(self, mom, vdf) -> float:
        """``||A f - b|| / ||b||`` in the solid-angle-weighted L2 norm, no sweep."""
        ts, _ = self._dev(mom.ts)
        qxs, _ = self._dev(mom.qxs)
        qys, _ = self._dev(mom.qys)
        v, _ = self._dev(vdf)
        _lib.check(_lib.lib().pbte_transport_residual(
            self._ctx, ts.data_ptr(), qxs.data_ptr(), qys.data_ptr(), v.data_ptr(),
            self.flux_wall.data_ptr(), self.pbuf.data_ptr(), self._num.data_ptr(),
            self._den.data_ptr(), _stream()), "pbte_transport_residual")
        d = float(self._den.sum().item())
        return float("nan") if d <= 0.0 else float(np.sqrt(float(self._num.sum().item()) / d))

    # -- the other device kernels --------------------------------------------
    def moments(self, vdf, mom: Moments, stream=None) -> Moments:
        fn = _lib.lib().pbte_moments if vdf.dtype == torch.float64 else _lib.lib().pbte_moments_f32
        _lib.check(fn(self._ctx, vdf.data_ptr(), mom.ts.data_ptr(), mom.qxs.data_ptr(),
                      mom.qys.data_ptr(), mom.temp.data_ptr(), mom.qx.data_ptr(),
                      mom.qy.data_ptr(), _stream(stream)), "pbte_moments")
        return mom

    def wall_flux(self, vdf, out=None, stream=None) -> None:
        out = self.flux_wall if out is None else out
        fn = _lib.lib().pbte_wall_flux if vdf.dtype == torch.float64 else _lib.lib().pbte_wall_flux_f32
        _lib.check(fn(self._ctx, vdf.data_ptr(), out.data_ptr(), _stream(stream)), "pbte_wall_flux")

    def sweep_f32(self, mom_or_state, vdf32, flux_wall, wall_scale: float = 1.0, stream=None) -> None:
        ts, qxs, qys = mom_or_state
        _lib.check(_lib.lib().pbte_sweep_f32(self._ctx, ts.data_ptr(), qxs.data_ptr(), qys.data_ptr(),
                                             vdf32.data_ptr(), flux_wall.data_ptr(), float(wall_scale),
                                             _stream(stream)), "pbte_sweep_f32")
