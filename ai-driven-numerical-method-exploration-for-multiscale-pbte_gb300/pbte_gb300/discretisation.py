"""Everything a case needs before the first sweep (pybte ``Solver.__init__``
steps 1-6, ``pybte/driver.py:61-80``): mesh, basis, ordinates, integral
tensors, boundary data -- plus the compact per-element description the GPU
sweep reads.

Compact sweep form.  For an affine triangle every per-element tensor of the
sweep is a scaling of a reference matrix:

* ``mass[:, :, i] = area2_i * ref_mass``
* ``gx[i] = area2_i (dxi_i0 ref_dx + dxi_i1 ref_dy)``, ``gy`` likewise
* ``fcm[i, il] = edge_scale_il * ref_edge[il]``, nonzero only on the
  ``(deg+1) x (deg+1)`` block of the DOFs on edge ``il``
* ``ttfc[i, il] = fcm[i, il] P``, with ``P`` picking, for each DOF of
  element ``i`` on edge ``il``, the neighbour DOF at the same point (the
  neighbour's other basis functions vanish on the shared edge).

So the sweep needs six small reference matrices plus ~20 numbers and one
gather map per element instead of ``9 N_p^2`` numbers per element.
:func:`check_compact_form` verifies the identities against the full tensors.
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np

from .basis import Basis, build_basis
from .bc import BoundaryData, build_boundary_data
from .config import Case
from .constants import BC_PERIODIC
from .integration import Integrals, build_integrals, edge_nodes
from .mesh import Mesh, build_mesh, load_raw
from .velocity import VelocityMesh, build_velocity_mesh

__all__ = ["Discretisation", "check_compact_form"]


@dataclass
class Discretisation:
    case: Case
    mesh: Mesh
    basis: Basis
    vel: VelocityMesh
    integrals: Integrals
    bcdata: BoundaryData
    edge_dofs: np.ndarray      # (3, nf)
    edge_map: np.ndarray       # (n_tris, 3, nf) upwind DOF facing each edge DOF, -1 on walls
    upwind_tri: np.ndarray     # (n_tris, 3) neighbour or periodic partner, -1 on walls

    @property
    def n_tris(self) -> int:
        return self.mesh.n_tris

    @property
    def ndof(self) -> int:
        return self.basis.ndof_tri

    @property
    def ndir(self) -> int:
        return self.vel.ndir

    @classmethod
    def build(cls, case: Case, raw=None) -> "Discretisation":
        c = case
        if not c.boundaries:
            raise ValueError("the case declares no boundaries")
        raw = raw if raw is not None else load_raw(c.mesh_path())
        xoff = [b.xoff for b in c.boundaries]
        yoff = [b.yoff for b in c.boundaries]
        mesh = build_mesh(raw, [b.phyid for b in c.boundaries], c.bc_codes(),
                          [b.name for b in c.boundaries], xoff, yoff)
        basis = build_basis(c.dg.deg)
        vel = build_velocity_mesh(c.velmesh.npole, c.velmesh.nazim, c.flow.vg)
        integrals = build_integrals(mesh, basis, c.np_fc, bc_codes=c.bc_codes(),
                                    bc_xoff=xoff, bc_yoff=yoff)
        bcdata = build_boundary_data(mesh, c.boundaries, c.ndof_tri)
        edofs = edge_nodes(c.dg.deg)
        upwind, emap = _edge_maps(mesh, basis, edofs, bcdata, np.asarray(c.bc_codes()),
                                  np.asarray(xoff, dtype=float), np.asarray(yoff, dtype=float))
        return cls(case=c, mesh=mesh, basis=basis, vel=vel, integrals=integrals,
                   bcdata=bcdata, edge_dofs=edofs, edge_map=emap, upwind_tri=upwind)


def _dof_positions(mesh: Mesh, basis: Basis, nodes=None) -> np.ndarray:
    nodes = mesh.nodes if nodes is None else nodes
    p = nodes[mesh.tri_nodes]                           # (n, 3, 2)
    xi = basis.node_tri[:, 0][None, :, None]
    eta = basis.node_tri[:, 1][None, :, None]
    return p[:, None, 0, :] + xi * (p[:, None, 1, :] - p[:, None, 0, :]) \
        + eta * (p[:, None, 2, :] - p[:, None, 0, :])


def _edge_maps(mesh: Mesh, basis: Basis, edofs, bcdata, bc_codes, xoff, yoff):
    n = mesh.n_tris
    nf = edofs.shape[1]
    pos = _dof_positions(mesh, basis)                   # (n, nd, 2)
    upwind = mesh.tri_neighbour.astype(np.int64).copy()
    shift = np.zeros((n, 3, 2))
    fb = mesh.face_bc[mesh.tri_faces]
    code = np.where(fb >= 0, bc_codes[np.clip(fb, 0, None)] if bc_codes.size else 0, 0)
    per = (fb >= 0) & (code == BC_PERIODIC)
    if per.any():
        ii, ll = np.nonzero(per)
        fc = mesh.tri_faces[ii, ll]
        upwind[ii, ll] = bcdata.periodic_tri[fc]
        # the partner's points shifted by the partner boundary's offset land on this face
        bcp = mesh.face_bc[mesh.face_pair[fc]]
        shift[ii, ll, 0] = xoff[bcp]
        shift[ii, ll, 1] = yoff[bcp]
    emap = np.full((n, 3, nf), -1, dtype=np.int64)
    h = float(np.min(mesh.face_len))
    for il in range(3):
        has = upwind[:, il] >= 0
        ids = np.flatnonzero(has)
        if ids.size == 0:
            continue
        mine = pos[ids][:, edofs[il], :]                               # (k, nf, 2)
        theirs = pos[upwind[ids, il]] + shift[ids, il][:, None, :]     # (k, nd, 2)
        # squared distances: the partner node is the one that coincides
        dx = mine[:, :, None, 0] - theirs[:, None, :, 0]
        dy = mine[:, :, None, 1] - theirs[:, None, :, 1]
        d2 = dx * dx + dy * dy
        best = d2.argmin(axis=-1)
        if np.sqrt(np.take_along_axis(d2, best[..., None], -1).max()) > 1e-8 * h:
            raise ValueError("non-conforming mesh: an edge node has no partner node "
                             "in the neighbouring element")
        emap[ids, il] = best
    return upwind.astype(np.int32), emap.astype(np.int32)


def check_compact_form(disc: Discretisation) -> dict:
    """Max relative deviation of each full tensor from its compact form."""
    it = disc.integrals
    nd = disc.ndof
    e = disc.edge_dofs
    out = {}
    mass = it.area2[None, None, :] * it.ref_mass[:, :, None]
    out["mass"] = float(np.abs(mass - it.int_tri_tri).max() / np.abs(it.int_tri_tri).max())
    fcm_block = np.zeros_like(it.int_tri_fc)
    for il in range(3):
        blk = it.ref_edge[il][np.ix_(e[il], e[il])]
        fcm_block[:, il][:, e[il][:, None], e[il][None, :]] = \
            it.edge_scale[:, il, None, None] * blk[None]
    out["fcm_block"] = float(np.abs(fcm_block - it.int_tri_fc).max() / np.abs(it.int_tri_fc).max())
    tt = np.zeros_like(it.int_tri_tri_fc)
    for il in range(3):
        has = disc.upwind_tri[:, il] >= 0
        ids = np.flatnonzero(has)
        for a, k in enumerate(e[il]):
            for b, kk in enumerate(e[il]):
                cols = disc.edge_map[ids, il, b]
                tt[ids, il, k, cols] += it.edge_scale[ids, il] * it.ref_edge[il][k, kk]
        wall = np.flatnonzero(~has)
        rs = it.ref_edge[il][np.ix_(e[il], e[il])].sum(axis=1)
        for a, k in enumerate(e[il]):
            tt[wall, il, k, :] = (it.edge_scale[wall, il] * rs[a])[:, None]
    out["ttfc"] = float(np.abs(tt - it.int_tri_tri_fc).max() / np.abs(it.int_tri_tri_fc).max())
    _ = nd
    return out
