"""Triangle meshes: the structured unit-square generator, a gmsh 2.2 reader, and
the face topology / element geometry the solver needs.

Face numbering and the ``(+)/(-)`` triangle of each face follow
``pybte/mesh/topology.py:333-482``: line elements create faces in file order,
then every triangle edge not yet seen creates a face oriented as that
triangle walks it.  Geometry follows ``pybte/mesh/geometry.py:32-86``
(edge ``j`` runs from node ``j`` to node ``j+1``; outward normal
``(-dy, dx)/L`` with ``(dx, dy) = p_j - p_{j+1}``).

The structured square reproduces the node numbering, boundary-line order and
per-quadrant diagonal choice of ``solver-python/tools/make_meshes.py:60-140``
(the benchmark meshes), including the 16-decimal rounding of the coordinates
that a round trip through the text file applies.
"""
from __future__ import annotations

from dataclasses import dataclass
from pathlib import Path

import numpy as np

from .constants import BC_SYMMETRY, BC_THERMALISING

__all__ = ["RawMesh", "Mesh", "structured_square", "read_gmsh22", "gmsh_text",
           "build_mesh"]


@dataclass
class RawMesh:
    """Element list as a gmsh file holds it (0-based node ids)."""
    nodes: np.ndarray        # (n_nodes, 2)
    line_nodes: np.ndarray   # (n_lines, 2)
    line_phyid: np.ndarray   # (n_lines,)
    tri_nodes: np.ndarray    # (n_tris, 3)
    #: position of each element in the file, lines and triangles interleaved
    #: only matters when they are; the generator writes all lines first
    lines_first: bool = True


def _dist(t: np.ndarray, kind: str) -> np.ndarray:
    if kind == "uniform":
        return t
    if kind == "smootherstep":
        return t ** 3 * (10.0 - 15.0 * t + 6.0 * t ** 2)
    raise ValueError(f"unknown distribution {kind!r}")


def structured_square(n: int, layout: str = "cavity", distribution: str = "uniform",
                      distribution_x: str | None = None) -> RawMesh:
    """Unit square with ``n x n`` quads split in two (``2 n^2`` triangles).

    Physical ids: 11 south, 12 north, 13 east, 14 west.  ``layout='channel'``
    keeps every x-column identical (diagonal flips on y only)."""
    if layout not in ("cavity", "channel"):
        raise ValueError(f"unknown layout {layout!r}")
    nn = n + 1
    t = np.arange(nn) / n
    cy = np.array([float(f"{v:.16f}") for v in _dist(t, distribution)])
    cx = np.array([float(f"{v:.16f}") for v in _dist(t, distribution_x or distribution)])
    ii, jj = np.meshgrid(np.arange(nn), np.arange(nn), indexing="ij")
    nodes = np.stack([cx[ii.ravel()], cy[jj.ravel()]], axis=1)

    def nid(i, j):
        return i * nn + j

    r = np.arange(n)
    south = np.stack([nid(r, 0), nid(r + 1, 0)], 1)
    north = np.stack([nid(n - r, n), nid(n - r - 1, n)], 1)
    east = np.stack([nid(n, r), nid(n, r + 1)], 1)
    west = np.stack([nid(0, n - r), nid(0, n - r - 1)], 1)
    line_nodes = np.concatenate([south, north, east, west]).astype(np.int64)
    line_phyid = np.repeat(np.array([11, 12, 13, 14]), n)

    I, J = np.meshgrid(r, r, indexing="ij")
    I = I.ravel()
    J = J.ravel()
    flip_x = (2 * I >= n) if layout == "cavity" else np.zeros_like(I, dtype=bool)
    diag_a = flip_x == (2 * J >= n)
    t1 = np.where(diag_a[:, None],
                  np.stack([nid(I, J), nid(I + 1, J), nid(I + 1, J + 1)], 1),
                  np.stack([nid(I, J), nid(I + 1, J), nid(I, J + 1)], 1))
    t2 = np.where(diag_a[:, None],
                  np.stack([nid(I, J), nid(I + 1, J + 1), nid(I, J + 1)], 1),
                  np.stack([nid(I, J + 1), nid(I + 1, J), nid(I + 1, J + 1)], 1))
    tri_nodes = np.stack([t1, t2], 1).reshape(-1, 3).astype(np.int64)
    return RawMesh(nodes=nodes, line_nodes=line_nodes, line_phyid=line_phyid,
                   tri_nodes=tri_nodes)


def gmsh_text(raw: RawMesh) -> str:
    """Render a mesh as gmsh 2.2 ASCII (all lines before all triangles)."""
    out = ["$MeshFormat\n2.2 0 8\n$EndMeshFormat\n$Nodes\n",
           f"{raw.nodes.shape[0]:6d}\n"]
    out += [f"{k + 1:6d} {x:.16f} {y:.16f} 0\n" for k, (x, y) in enumerate(raw.nodes)]
    out.append("$EndNodes\n$Elements\n")
    nl = raw.line_nodes.shape[0]
    out.append(f"{nl + raw.tri_nodes.shape[0]:6d}\n")
    for k in range(nl):
        a, b = raw.line_nodes[k] + 1
        out.append(f"{k + 1:6d} 1 2 {raw.line_phyid[k]} 0 {a:5d} {b:5d}\n")
    for k, (a, b, c) in enumerate(raw.tri_nodes + 1):
        out.append(f"{nl + k + 1:6d} 2 2 15 10 {a:5d} {b:5d} {c:5d}\n")
    out.append("$EndElements\n")
    return "".join(out)


def read_gmsh22(path) -> RawMesh:
    """gmsh 2.2 ASCII: ``$Nodes`` and line/triangle ``$Elements`` only
    (``pybte/mesh/gmsh_reader.py:131-208``); rejects other element types,
    fewer than two tags, and node ids that are not ``1..N`` in order."""
    path = Path(path)
    lines = path.read_text().splitlines()
    i = 0
    nodes = None
    lnodes, lphy, tnodes, order = [], [], [], []
    while i < len(lines):
        tag = lines[i].strip()
        if tag == "$MeshFormat":
            ver = lines[i + 1].split()
            if not ver[0].startswith("2.2") or ver[1] != "0":
                raise ValueError(f"{path}: expected gmsh ASCII 2.2")
            i += 2
        elif tag == "$Nodes":
            cnt = int(lines[i + 1])
            arr = np.array([lines[i + 2 + k].split()[:3] for k in range(cnt)], dtype=np.float64)
            if not np.array_equal(arr[:, 0], np.arange(1, cnt + 1)):
                raise ValueError(f"{path}: node ids are not 1..{cnt} in order")
            nodes = arr[:, 1:3].copy()
            i += 2 + cnt
        elif tag == "$Elements":
            cnt = int(lines[i + 1])
            for k in range(cnt):
                p = lines[i + 2 + k].split()
                etype, ntags = int(p[1]), int(p[2])
                if etype not in (1, 2):
                    raise ValueError(f"{path}: element {p[0]} has unsupported type {etype}")
                if ntags < 2:
                    raise ValueError(f"{path}: element {p[0]} has {ntags} tags, need >= 2")
                nds = [int(v) - 1 for v in p[3 + ntags:3 + ntags + (2 if etype == 1 else 3)]]
                if etype == 1:
                    lnodes.append(nds)
                    lphy.append(int(p[3]))
                    order.append(0)
                else:
                    tnodes.append(nds)
                    order.append(1)
            i += 2 + cnt
        else:
            i += 1
    if nodes is None:
        raise ValueError(f"{path}: no $Nodes section")
    if not tnodes:
        raise ValueError(f"{path}: no triangles")
    order = np.asarray(order)
    first_tri = int(np.argmax(order == 1))
    lines_first = not np.any(order[first_tri:] == 0)
    return RawMesh(nodes=nodes, line_nodes=np.asarray(lnodes, dtype=np.int64).reshape(-1, 2),
                   line_phyid=np.asarray(lphy, dtype=np.int64),
                   tri_nodes=np.asarray(tnodes, dtype=np.int64), lines_first=lines_first)


@dataclass
class Mesh:
    """Topology and geometry (0-based, -1 = absent); field meanings as in
    ``pybte/mesh/topology.py:240-277``."""
    nodes: np.ndarray
    tri_nodes: np.ndarray
    tri_faces: np.ndarray
    tri_area: np.ndarray
    tri_normal: np.ndarray
    tri_hmin: np.ndarray
    hmin: float
    face_nodes: np.ndarray
    face_bc: np.ndarray
    face_pair: np.ndarray
    face_tri: np.ndarray
    face_lfc: np.ndarray
    face_len: np.ndarray
    tri_neighbour: np.ndarray
    bc_codes: np.ndarray

    @property
    def n_tris(self) -> int:
        return self.tri_nodes.shape[0]

    @property
    def n_faces(self) -> int:
        return self.face_nodes.shape[0]

    @property
    def n_faces_b(self) -> int:
        return int(np.count_nonzero(self.face_bc >= 0))

    def adjacent(self, face: int):
        """(triangle, local edge) of the element on a boundary face, (+) first."""
        if self.face_tri[face, 0] < 0:
            return int(self.face_tri[face, 1]), int(self.face_lfc[face, 1])
        return int(self.face_tri[face, 0]), int(self.face_lfc[face, 0])

    def adjacent_all(self) -> tuple[np.ndarray, np.ndarray]:
        """Vectorised :meth:`adjacent` for every face."""
        use_minus = self.face_tri[:, 0] < 0
        tri = np.where(use_minus, self.face_tri[:, 1], self.face_tri[:, 0])
        lfc = np.where(use_minus, self.face_lfc[:, 1], self.face_lfc[:, 0])
        return tri, lfc


def _geometry(nodes, tri_nodes):
    x = nodes[tri_nodes, 0]
    y = nodes[tri_nodes, 1]
    x1, x2, x3 = x[:, 0], x[:, 1], x[:, 2]
    y1, y2, y3 = y[:, 0], y[:, 1], y[:, 2]
    area = 0.5 * (x3 * y1 - x2 * y1 + x1 * y2 - x3 * y2 - x1 * y3 + x2 * y3)
    if np.any(area < 0):
        raise ValueError(f"{int(np.count_nonzero(area < 0))} triangles have negative area")
    dx = x - np.roll(x, -1, axis=1)
    dy = y - np.roll(y, -1, axis=1)
    length = np.sqrt(dx * dx + dy * dy)
    normal = np.stack([-dy / length, dx / length], axis=-1)
    hl = 2.0 * area[:, None] / length
    return area, normal, hl.min(axis=1), min(1.0, float(hl.min()))


def _edge_key(p: np.ndarray) -> list:
    """Orientation-free keys of edges given by their end points ``p`` (k, 2, 2):
    the two ends ordered lexicographically, as a tuple of four floats (equal
    coordinates compare equal, -0.0 included)."""
    x0, y0, x1, y1 = p[:, 0, 0], p[:, 0, 1], p[:, 1, 0], p[:, 1, 1]
    keep = (x0 < x1) | ((x0 == x1) & (y0 <= y1))
    lo = np.where(keep[:, None], p[:, 0], p[:, 1])
    hi = np.where(keep[:, None], p[:, 1], p[:, 0])
    return list(map(tuple, np.concatenate([lo, hi], axis=1).tolist()))


def _pair_master_slave(nodes, face_nodes, face_bc, bc_names, bc_xoff, bc_yoff) -> np.ndarray:
    """Periodic partners of the boundaries named ``Master`` and ``Slave``
    (``pybte/mesh/topology.py:186-209``): a Master face, moved by the Master
    boundary's offset, pairs with the Slave face that has exactly the same two
    end points, in either order; the lowest-numbered such Slave face wins.
    A hash join over orientation-free edge keys, linear in the face count."""
    n_faces = face_nodes.shape[0]
    face_pair = np.full(n_faces, -1, dtype=np.int32)
    names = [str(s).strip() for s in bc_names]
    if "Master" not in names:
        return face_pair
    if "Slave" not in names:
        raise ValueError("a 'Master' boundary needs a matching 'Slave'")
    bm, bs = names.index("Master"), names.index("Slave")
    masters = np.flatnonzero(face_bc == bm)
    slaves = np.flatnonzero(face_bc == bs)
    shift = np.array([bc_xoff[bm], bc_yoff[bm]])
    by_key = {}
    for s, key in zip(slaves[::-1].tolist(), _edge_key(nodes[face_nodes[slaves[::-1]]])):
        by_key[key] = s
    for m, key in zip(masters.tolist(), _edge_key(nodes[face_nodes[masters]] + shift)):
        s = by_key.get(key)
        if s is not None:
            face_pair[m] = s
            face_pair[s] = m
    lonely = np.concatenate([masters, slaves])
    lonely = lonely[face_pair[lonely] < 0]
    if lonely.size:
        raise ValueError(f"periodic faces without a partner: {lonely[:8].tolist()}")
    return face_pair


def build_mesh(raw: RawMesh, bc_phyid, bc_codes, bc_names=None,
               bc_xoff=None, bc_yoff=None) -> Mesh:
    """Faces, connectivity, periodic pairing and geometry from a raw mesh."""
    if not raw.lines_first:
        raise ValueError("interleaved line/triangle elements are not supported")
    nbc = len(bc_phyid)
    bc_phyid = np.asarray(bc_phyid, dtype=np.int64)
    bc_codes = np.asarray(bc_codes, dtype=np.int64)
    bc_names = list(bc_names) if bc_names is not None else [""] * nbc
    bc_xoff = np.asarray(bc_xoff if bc_xoff is not None else np.zeros(nbc), dtype=float)
    bc_yoff = np.asarray(bc_yoff if bc_yoff is not None else np.zeros(nbc), dtype=float)
    nodes = raw.nodes
    nn = np.int64(nodes.shape[0])
    tri_nodes = raw.tri_nodes.astype(np.int64)
    n_tris = tri_nodes.shape[0]

    # boundary lines: a face each; the last matching BC id wins
    lb = np.full(raw.line_nodes.shape[0], -1, dtype=np.int64)
    for j in range(nbc):
        lb[raw.line_phyid == bc_phyid[j]] = j
    la, lbn = raw.line_nodes[:, 0], raw.line_nodes[:, 1]
    lkey = np.minimum(la, lbn) * nn + np.maximum(la, lbn)
    if np.unique(lkey).size != lkey.size:
        raise ValueError("duplicate boundary edge")

    # triangle edges in (triangle, local edge) order
    ea = tri_nodes
    eb = np.roll(tri_nodes, -1, axis=1)
    ekey = (np.minimum(ea, eb) * nn + np.maximum(ea, eb)).ravel()
    uk, first = np.unique(ekey, return_index=True)
    is_line = np.isin(uk, lkey)
    new = np.sort(first[~is_line])
    n_lines = lkey.size
    face_key = np.concatenate([lkey, ekey[new]])
    face_nodes = np.concatenate([raw.line_nodes,
                                 np.stack([ea.ravel()[new], eb.ravel()[new]], 1)]).astype(np.int32)
    face_bc = np.concatenate([lb, np.full(new.size, -1)]).astype(np.int32)
    n_faces = face_key.size
    srt = np.argsort(face_key)
    pos = np.searchsorted(face_key[srt], ekey)
    tri_faces = srt[pos].reshape(n_tris, 3).astype(np.int32)

    plus = (face_nodes[tri_faces, 0] == ea) & (face_nodes[tri_faces, 1] == eb)
    face_tri = np.full((n_faces, 2), -1, dtype=np.int32)
    face_lfc = np.full((n_faces, 2), -1, dtype=np.int32)
    ti = np.repeat(np.arange(n_tris), 3).reshape(n_tris, 3)
    lj = np.tile(np.arange(3), (n_tris, 1))
    for side, sel in ((0, plus), (1, ~plus)):
        face_tri[tri_faces[sel], side] = ti[sel]
        face_lfc[tri_faces[sel], side] = lj[sel]

    other = np.where(face_tri[tri_faces, 0] == ti, face_tri[tri_faces, 1], face_tri[tri_faces, 0])
    tri_neighbour = other.astype(np.int32)

    face_pair = _pair_master_slave(nodes, face_nodes, face_bc, bc_names, bc_xoff, bc_yoff)
    counter = 0
    for k in np.flatnonzero(face_bc >= 0):
        if bc_codes[face_bc[k]] in (BC_THERMALISING, BC_SYMMETRY):
            face_pair[k] = counter
            counter += 1

    area, normal, hmin_tri, hmin = _geometry(nodes, tri_nodes)
    fn = nodes[face_nodes]
    d = fn[:, 0, :] - fn[:, 1, :]
    face_len = np.sqrt(d[:, 0] * d[:, 0] + d[:, 1] * d[:, 1])

    mesh = Mesh(nodes=nodes, tri_nodes=tri_nodes.astype(np.int32), tri_faces=tri_faces,
                tri_area=area, tri_normal=normal, tri_hmin=hmin_tri, hmin=hmin,
                face_nodes=face_nodes, face_bc=face_bc, face_pair=face_pair,
                face_tri=face_tri, face_lfc=face_lfc, face_len=face_len,
                tri_neighbour=tri_neighbour, bc_codes=bc_codes)
    interior = face_bc < 0
    if np.any((face_tri[interior] < 0).any(axis=1)):
        raise ValueError("interior faces with a missing neighbour (hole or untagged boundary)")
    if np.any((face_tri[~interior] >= 0).all(axis=1)):
        raise ValueError("boundary faces with two neighbours")
    _ = n_lines
    return mesh


def load_raw(spec) -> RawMesh:
    """``"cavity:N[:dist]"`` / ``"channel:N[:dist]"`` (structured square,
    ``dist`` = ``uniform`` (default) or ``smootherstep`` grading in y -- and in
    x for the cavity) or a gmsh 2.2 path."""
    s = str(spec)
    if ":" in s and s.split(":")[0] in ("cavity", "channel"):
        parts = s.split(":")
        kind, n = parts[0], int(parts[1])
        dist = parts[2] if len(parts) > 2 else "uniform"
        if kind == "channel":
            return structured_square(n, "channel", dist, "uniform")
        return structured_square(n, "cavity", dist)
    return read_gmsh22(s)
