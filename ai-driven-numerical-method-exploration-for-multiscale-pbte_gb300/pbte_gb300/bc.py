"""Boundary data (``pybte/bc.py:327-460``).

Wall types, as dispatched by the sweep: 1 thermalising (inflow
``cv T_w / 4 pi``), 2 non-thermalising (diffuse re-emission that zeroes the
net normal flux, ``flux_wall`` refreshed from the previous iterate),
3 periodic (inflow from the partner element), 4 symmetry (rejected).
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np

from .constants import BC_NONTHERMALISING, BC_PERIODIC, BC_SYMMETRY

__all__ = ["BoundaryData", "build_boundary_data"]


@dataclass
class BoundaryData:
    bc_type: np.ndarray        # (nbc,) int32
    bc_temp: np.ndarray        # (nbc,)
    periodic_tri: np.ndarray   # (n_faces,) int32, element behind the pair or -1
    periodic_flip: np.ndarray  # (n_faces,) bool
    flux_wall: np.ndarray      # (n_faces, ndof) host copy of the wall emission
    has_nonthermalising: bool
    has_periodic: bool


def build_boundary_data(mesh, boundaries, ndof_tri: int) -> BoundaryData:
    bc_type = np.array([b.code for b in boundaries], dtype=np.int32)
    bc_temp = np.array([float(b.temp) for b in boundaries], dtype=np.float64)
    bc_xoff = np.array([float(b.xoff) for b in boundaries], dtype=np.float64)
    bc_yoff = np.array([float(b.yoff) for b in boundaries], dtype=np.float64)
    if np.any(bc_type == BC_SYMMETRY):
        raise NotImplementedError("symmetry walls (type 4) are not implemented; "
                                  "use a periodic pair instead")
    n_faces = mesh.n_faces
    periodic_tri = np.full(n_faces, -1, dtype=np.int32)
    periodic_flip = np.zeros(n_faces, dtype=bool)
    has_periodic = bool(np.any(bc_type == BC_PERIODIC))
    if has_periodic:
        for f in np.flatnonzero(mesh.face_bc >= 0):
            bc = int(mesh.face_bc[f])
            if bc_type[bc] != BC_PERIODIC:
                continue
            pair = int(mesh.face_pair[f])
            if pair < 0:
                raise ValueError(f"periodic face {f} has no partner")
            periodic_tri[f] = mesh.adjacent(pair)[0]
            a = mesh.nodes[mesh.face_nodes[f, 0]] + np.array([bc_xoff[bc], bc_yoff[bc]])
            b1 = mesh.nodes[mesh.face_nodes[pair, 0]]
            b2 = mesh.nodes[mesh.face_nodes[pair, 1]]
            if np.allclose(a, b2) and not np.allclose(a, b1):
                periodic_flip[f] = True
            elif not np.allclose(a, b1):
                raise ValueError(f"periodic faces {f} and {pair} do not line up")
    return BoundaryData(bc_type=bc_type, bc_temp=bc_temp, periodic_tri=periodic_tri,
                        periodic_flip=periodic_flip,
                        flux_wall=np.zeros((n_faces, ndof_tri)),
                        has_nonthermalising=bool(np.any(bc_type == BC_NONTHERMALISING)),
                        has_periodic=has_periodic)
