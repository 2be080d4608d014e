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


def _wall_table(boundaries):
    """Per boundary condition: code, wall temperature and periodic offset."""
    code = np.fromiter((b.code for b in boundaries), dtype=np.int32, count=len(boundaries))
    temp = np.fromiter((float(b.temp) for b in boundaries), dtype=np.float64, count=len(boundaries))
    shift = np.array([[float(b.xoff), float(b.yoff)] for b in boundaries], dtype=np.float64).reshape(-1, 2)
    return code, temp, shift


def _periodic_links(mesh, code, shift):
    """For every face of a periodic pair: the element behind its partner face,
    and whether the partner's 1-D trace runs the opposite way (its first node
    matches this face's first node only after the pair's shift when the two
    faces are walked in the same sense; otherwise their DOFs are mirrored).

    All periodic faces are treated at once: each face's first node, shifted
    by its boundary's offset, is compared with both end nodes of the partner,
    with the tolerance of ``numpy.allclose`` per coordinate pair."""
    n = mesh.n_faces
    behind = np.full(n, -1, dtype=np.int32)
    mirrored = np.zeros(n, dtype=bool)
    fb = mesh.face_bc
    wall = fb >= 0
    is_pair = np.zeros(n, dtype=bool)
    is_pair[wall] = code[fb[wall]] == BC_PERIODIC
    faces = np.flatnonzero(is_pair)
    if faces.size == 0:
        return behind, mirrored
    partner = mesh.face_pair[faces]
    lonely = faces[partner < 0]
    if lonely.size:
        raise ValueError(f"periodic face {int(lonely[0])} has no partner face "
                         f"({lonely.size} periodic faces without one)")
    tri_of_face, _ = mesh.adjacent_all()
    behind[faces] = tri_of_face[partner]
    first = mesh.nodes[mesh.face_nodes[faces, 0]] + shift[fb[faces]]
    ends = mesh.nodes[mesh.face_nodes[partner]]                  # (k, 2 ends, 2 coords)
    same_sense = np.isclose(first, ends[:, 0]).all(axis=1)
    reversed_sense = np.isclose(first, ends[:, 1]).all(axis=1)
    misfit = ~(same_sense | reversed_sense)
    if misfit.any():
        f = int(faces[misfit][0])
        raise ValueError(f"periodic face {f} and its partner {int(mesh.face_pair[f])} do not meet "
                         f"under the boundary's offset {tuple(shift[fb[f]])}")
    mirrored[faces] = reversed_sense & ~same_sense
    return behind, mirrored


def build_boundary_data(mesh, boundaries, ndof_tri: int) -> BoundaryData:
    """Wall tables and periodic links for the sweep (``pybte/bc.py:120-170``):
    symmetry walls are refused, as pybte does, since its transport solve never
    implements them."""
    code, temp, shift = _wall_table(boundaries)
    if (code == BC_SYMMETRY).any():
        raise NotImplementedError("symmetry walls (type 4) have no transport treatment; "
                                  "describe the domain with a periodic pair instead")
    behind, mirrored = _periodic_links(mesh, code, shift)
    return BoundaryData(bc_type=code, bc_temp=temp, periodic_tri=behind, periodic_flip=mirrored,
                        flux_wall=np.zeros((mesh.n_faces, ndof_tri)),
                        has_nonthermalising=bool((code == BC_NONTHERMALISING).any()),
                        has_periodic=bool((code == BC_PERIODIC).any()))
