"""Field output and run-log writers behind pybte's ``io_output`` interface
(``pybte/io_output.py:166-308``).

``locate_points`` and ``sample_fields`` run on the GPU through the C ABI
(``pbte_locate_points``, ``pbte_field_moments``, ``pbte_sample_fields``);
the sampling grid and the two text writers are host formatting, byte for
byte the reference's file formats:

``sampling_grid``       the 109 x 109 grid clustered at the walls
                        (``io_output.py:167-184``);
``write_tecplot``       point-ordered Tecplot ASCII (``io_output.py:279-291``);
``append_runtime_log``  one ``RunTime.txt`` line per run, Fortran
                        ``FORMAT(1X,A4,2ES10.2,3I6,I8,F20.1)``
                        (``io_output.py:294-308``).
"""
from __future__ import annotations

import math
from pathlib import Path

import numpy as np
import torch

from . import _lib

__all__ = ["sampling_grid", "locate_points", "sample_fields", "write_tecplot",
           "append_runtime_log", "PointBins"]


def sampling_grid(nx: int = 109, ny: int = 109):
    """``(px, py)``.  For the default 109 x 109: five smootherstep-clustered
    points inside each outer 2 % of [0, 1] and 99 uniform points between
    (``io_output.py:167-184``); any other size is a uniform ``linspace``."""
    if nx == 109 and ny == 109:
        a = np.arange(5) / 8.0
        edge = a * a * a * (10.0 - 15.0 * a + 6.0 * a * a) * 0.02
        mid = (np.arange(6, 105) - 5.0) * (1.0 - 0.02) / 100.0 + 0.01
        g = np.concatenate([edge, mid, (1.0 - edge)[::-1]])
        return g.copy(), g
    return np.linspace(0.0, 1.0, nx), np.linspace(0.0, 1.0, ny)


def _tri_xy(mesh) -> tuple[np.ndarray, np.ndarray]:
    tn = np.asarray(mesh.tri_nodes)
    return (np.ascontiguousarray(mesh.nodes[tn, 0], dtype=np.float64),
            np.ascontiguousarray(mesh.nodes[tn, 1], dtype=np.float64))


class PointBins:
    """Uniform bin grid over a mesh's elements for ``pbte_locate_points``.

    An element is listed, in increasing index, in every bin its box touches
    once widened past the point-in-triangle slack: a sub-area
    ``0.5 |e| dist >= -1e-12`` admits points up to ``2e-12 / |e|`` outside
    edge ``e`` (plus rounding of the products, bounded by the coordinates'
    magnitude), and a corner of opening angle ``theta`` moves
    ``1 / sin(theta / 2)`` times further than its edges.  A point's bin is
    computed with the same IEEE operations on both sides, so every element
    the scan could accept is among its bin's candidates."""

    def __init__(self, tx: np.ndarray, ty: np.ndarray, bins_per_side: int | None = None):
        nt = tx.shape[0]
        lo_x, hi_x = float(tx.min()), float(tx.max())
        lo_y, hi_y = float(ty.min()), float(ty.max())
        nb = bins_per_side or int(min(max(math.ceil(math.sqrt(nt)), 1), 2048))
        self.nbx = self.nby = nb
        self.x0, self.y0 = lo_x, lo_y
        self.hx = (hi_x - lo_x) / nb if hi_x > lo_x else 1.0
        self.hy = (hi_y - lo_y) / nb if hi_y > lo_y else 1.0
        ex = np.roll(tx, -1, axis=1) - tx
        ey = np.roll(ty, -1, axis=1) - ty
        elen = np.hypot(ex, ey)                                 # (nt, 3) edge il -> il+1
        scale = max(abs(lo_x), abs(hi_x), abs(lo_y), abs(hi_y), 1.0)
        slack = (2e-12 + 64 * np.finfo(float).eps * scale * scale) / np.maximum(elen.min(axis=1), 1e-300)
        # interior angle at each corner from its two edges
        cosang = -(ex * np.roll(ex, 1, axis=1) + ey * np.roll(ey, 1, axis=1)) / np.maximum(
            elen * np.roll(elen, 1, axis=1), 1e-300)
        ang = np.arccos(np.clip(cosang, -1.0, 1.0)).min(axis=1)
        grow = 2.0 * slack / np.maximum(np.sin(0.5 * ang), 1e-12) + 1e-12 * scale

        def cell(v, v0, h):
            return np.clip(np.floor((v - v0) / h), 0, nb - 1).astype(np.int64)

        cx0 = cell(tx.min(axis=1) - grow, self.x0, self.hx)
        cx1 = cell(tx.max(axis=1) + grow, self.x0, self.hx)
        cy0 = cell(ty.min(axis=1) - grow, self.y0, self.hy)
        cy1 = cell(ty.max(axis=1) + grow, self.y0, self.hy)
        wx, wy = cx1 - cx0 + 1, cy1 - cy0 + 1
        cnt = wx * wy
        elem = np.repeat(np.arange(nt, dtype=np.int64), cnt)
        off = np.arange(elem.size, dtype=np.int64) - np.repeat(np.cumsum(cnt) - cnt, cnt)
        bx = cx0[elem] + off // wy[elem]
        by = cy0[elem] + off % wy[elem]
        b = bx * nb + by
        order = np.argsort(b, kind="stable")                   # keeps element order within a bin
        self.items = elem[order].astype(np.int32)
        self.start = np.zeros(nb * nb + 1, dtype=np.int32)
        np.cumsum(np.bincount(b, minlength=nb * nb), out=self.start[1:])

    def cell_of(self, x: np.ndarray, y: np.ndarray) -> np.ndarray:
        """Bin index of points, as the kernel computes it."""
        cx = np.clip(np.floor((x - self.x0) / self.hx), 0, self.nbx - 1).astype(np.int64)
        cy = np.clip(np.floor((y - self.y0) / self.hy), 0, self.nby - 1).astype(np.int64)
        return cx * self.nby + cy


def _dev(device):
    d = torch.device(device if device is not None else "cuda")
    if d.type != "cuda" or not torch.cuda.is_available():
        raise RuntimeError("field output runs on the GPU; there is no CPU fallback")
    return d


def _t(a, dev, dtype=torch.float64):
    return torch.as_tensor(np.ascontiguousarray(a), dtype=dtype).to(dev)


def locate_points(mesh, px, py, device=None, bins: PointBins | None = None) -> np.ndarray:
    """``(nx, ny)`` int32 array of containing element ids, ``-1`` outside
    (``io_output.py:187-217``): pybte's sub-area test with its ``-1e-12``
    slack and first-match-wins order, on the GPU."""
    dev = _dev(device)
    px = np.asarray(px, dtype=np.float64).ravel()
    py = np.asarray(py, dtype=np.float64).ravel()
    tx, ty = _tri_xy(mesh)
    bins = bins if bins is not None else PointBins(tx, ty)
    d_tx, d_ty, d_px, d_py = (_t(a, dev) for a in (tx, ty, px, py))
    d_start, d_items = _t(bins.start, dev, torch.int32), _t(bins.items, dev, torch.int32)
    out = torch.empty(px.size * py.size, dtype=torch.int32, device=dev)
    s = torch.cuda.current_stream(dev).cuda_stream
    _lib.check(_lib.lib().pbte_locate_points(
        d_tx.data_ptr(), d_ty.data_ptr(), tx.shape[0], bins.x0, bins.y0, bins.hx, bins.hy, bins.nbx,
        bins.nby, d_start.data_ptr(), d_items.data_ptr(), d_px.data_ptr(), px.size, d_py.data_ptr(),
        py.size, out.data_ptr(), s), "locate_points")
    return out.cpu().numpy().reshape(px.size, py.size)


def sample_fields(mesh, basis, vdf, cxv, cyv, domega, cv, px, py, triid, uq=None, ndof_tri=None,
                  device=None):
    """``(T, qx, qy, Nxx, Nxy, Nyy)`` on the ``(nx, ny)`` grid
    (``io_output.py:220-276``).  ``vdf`` ``(ndir, n_tris, ndof)`` and ``uq``
    ``(7 ndof, n_tris)`` may be device tensors (used in place) or host
    arrays; the stress trio is zero without ``uq``."""
    if isinstance(vdf, torch.Tensor):
        dev = _dev(vdf.device if device is None else device)
        d_vdf = vdf.to(dev, torch.float64).contiguous()
    else:
        dev = _dev(device)
        d_vdf = _t(vdf, dev)
    ndir, nt, nd_v = d_vdf.shape
    nd = basis.ndof_tri if ndof_tri is None else int(ndof_tri)
    if nd != nd_v:
        raise ValueError(f"vdf has {nd_v} DOFs per element, the basis {nd}")
    px = np.asarray(px, dtype=np.float64).ravel()
    py = np.asarray(py, dtype=np.float64).ravel()
    triid = np.asarray(triid, dtype=np.int32).reshape(-1)
    if triid.size != px.size * py.size:
        raise ValueError("triid does not match the grid")
    if triid.size and int(triid.max()) >= nt:
        raise ValueError("triid names an element past the mesh")
    cxv, cyv, domega = (np.asarray(a, dtype=np.float64) for a in (cxv, cyv, domega))
    w = [_t(a, dev) for a in (domega, cxv * domega, cyv * domega)]
    m = [torch.empty((nd, nt), dtype=torch.float64, device=dev) for _ in range(3)]
    s = torch.cuda.current_stream(dev).cuda_stream
    L = _lib.lib()
    _lib.check(L.pbte_field_moments(d_vdf.data_ptr(), ndir, nt, nd, *(a.data_ptr() for a in w),
                                    *(a.data_ptr() for a in m), s), "field_moments")
    tx, ty = _tri_xy(mesh)
    d_tx, d_ty, d_px, d_py = (_t(a, dev) for a in (tx, ty, px, py))
    d_tri = _t(triid, dev, torch.int32)
    d_nod = _t(basis.nodfun_tri, dev)
    d_mono = _t(np.asarray(basis.mono), dev, torch.int32)
    d_uq = None
    if uq is not None:
        d_uq = (uq.to(dev, torch.float64).contiguous() if isinstance(uq, torch.Tensor) else _t(uq, dev))
        if tuple(d_uq.shape) != (7 * nd, nt):
            raise ValueError(f"uq must be (7*ndof, n_tris) = {(7 * nd, nt)}")
    out = torch.empty((6, px.size * py.size), dtype=torch.float64, device=dev)
    _lib.check(L.pbte_sample_fields(d_tx.data_ptr(), d_ty.data_ptr(), d_tri.data_ptr(), d_px.data_ptr(), px.size,
                                    d_py.data_ptr(), py.size, d_nod.data_ptr(), d_mono.data_ptr(), nd,
                                    *(a.data_ptr() for a in m), nt, float(cv),
                                    d_uq.data_ptr() if d_uq is not None else None, out.data_ptr(), s),
               "sample_fields")
    h = out.cpu().numpy().reshape(6, px.size, py.size)
    return tuple(np.ascontiguousarray(h[q]) for q in range(6))


def write_tecplot(path, px, py, arrays, names) -> Path:
    """Tecplot ASCII, point order, x fastest (``io_output.py:279-291``)."""
    path = Path(path)
    path.parent.mkdir(parents=True, exist_ok=True)
    px, py = np.asarray(px), np.asarray(py)
    head = " VARIABLES=" + ",".join(f'"{n}"' for n in ["x", "y", *names]) + "\n"
    rows = [head, f" ZONE I = {px.size} J = {py.size}\n"]
    for j in range(py.size):
        for i in range(px.size):
            rows.append(" " + "".join(f"{v:16.6E}" for v in (px[i], py[j], *(a[i, j] for a in arrays))) + "\n")
    path.write_text("".join(rows))
    return path


def append_runtime_log(path, scheme, tau_r, tau_n, n_tris, npole, nazim, step, seconds) -> Path:
    """Append one ``RunTime.txt`` line (``io_output.py:294-308``).  Python's
    ``10.2E`` prints what Fortran's ``ES10.2`` does for any exponent of two
    digits, which every relaxation time has."""
    path = Path(path)
    path.parent.mkdir(parents=True, exist_ok=True)
    with path.open("a") as fh:
        fh.write(f" {scheme:>4s}{tau_r:10.2E}{tau_n:10.2E}{n_tris:6d}{npole:6d}{nazim:6d}{step:8d}{seconds:20.1f}\n")
    return path
