"""Setup arrays against the reference's own (golden fixtures made by
tests/golden/make_golden.py from pybte), and the compact-operator identities."""
import numpy as np
import pytest

from cases import golden, small_case
from pbte_gb300.discretisation import Discretisation, check_compact_form
from pbte_gb300.mesh import gmsh_text, read_gmsh22, structured_square
from pbte_gb300.velocity import build_velocity_mesh, twin_map


@pytest.mark.parametrize("deg", [1, 2, 3])
def test_setup_matches_reference(deg):
    z = golden(f"setup_sweep_deg{deg}")
    disc = Discretisation.build(small_case(deg, 4, 8, 0.5, 0.05))
    m, it = disc.mesh, disc.integrals
    for k in ("tri_nodes", "tri_faces", "face_nodes", "face_bc", "face_tri", "face_lfc"):
        assert np.array_equal(getattr(m, k), z[k]), k
    assert np.array_equal(m.tri_neighbour, z["tri_neighbour"])
    for k in ("nodes", "tri_normal", "tri_area", "face_len", "tri_hmin"):
        assert np.array_equal(getattr(m, k), z[k]), k
    cx, cy, dw = disc.vel.flat()
    assert np.array_equal(cx, z["cxv"]) and np.array_equal(cy, z["cyv"]) and np.array_equal(dw, z["domega"])
    for k in ("int_tri", "int_tri_tri", "int_tri_tri_x", "int_tri_tri_y", "int_tri_fc", "int_tri_fc_fc",
              "int_fc_fc", "int_fc", "int_tri_tri_fc"):
        a, b = getattr(it, k), z[k]
        assert a.shape == b.shape, k
        assert np.abs(a - b).max() <= 1e-13 * np.abs(b).max(), k


@pytest.mark.parametrize("deg", [1, 2, 3, 4])
def test_compact_form_identities(deg):
    disc = Discretisation.build(small_case(deg, 4, 8, 0.5, 0.05, mesh="cavity:4"))
    dev = check_compact_form(disc)
    # off-edge-block entries of the full tensors are rounding noise of the
    # monomial contraction; it grows with the basis conditioning (deg 4: 2e-12)
    tol = 1e-12 if deg < 4 else 1e-11
    assert dev["mass"] < 1e-14 and dev["fcm_block"] < tol and dev["ttfc"] < tol, dev


def test_gmsh_round_trip(tmp_path):
    raw = structured_square(7, "cavity", "smootherstep")
    p = tmp_path / "m.msh"
    p.write_text(gmsh_text(raw))
    back = read_gmsh22(p)
    assert np.array_equal(back.nodes, raw.nodes)
    assert np.array_equal(back.tri_nodes, raw.tri_nodes)
    assert np.array_equal(back.line_nodes, raw.line_nodes)


def test_gmsh_reader_rejects_bad_element(tmp_path):
    p = tmp_path / "bad.msh"
    p.write_text("$MeshFormat\n2.2 0 8\n$EndMeshFormat\n$Nodes\n1\n1 0 0 0\n$EndNodes\n"
                 "$Elements\n1\n1 15 2 1 1 1\n$EndElements\n")
    with pytest.raises(ValueError):
        read_gmsh22(p)


def test_ordinates_sum_to_4pi_and_have_z_twins():
    v = build_velocity_mesh(8, 32)
    cx, cy, dw = v.flat()
    # the reference's Newton quadrature leaves its weights ~1e-13 from exact
    assert abs(dw.sum() - 4 * np.pi) < 1e-10
    tw = twin_map(cx, cy, dw)
    assert np.all(tw != np.arange(cx.size))
    assert np.all(tw[tw] == np.arange(cx.size))


def test_square_counts():
    disc = Discretisation.build(small_case(2, 4, 8, 1.0, 0.1, mesh="cavity:64"))
    assert disc.n_tris == 8192 and disc.mesh.n_faces == 12416


def _edge_maps_brute_force(mesh, basis, edofs, bcdata, bc_codes, xoff, yoff):
    """Each edge node's partner: the nearest of all the neighbour's nodes
    (Euclidean norm), the partner's nodes shifted by a periodic offset."""
    from pbte_gb300.constants import BC_PERIODIC
    from pbte_gb300.discretisation import _dof_positions
    n, nf = mesh.n_tris, edofs.shape[1]
    pos = _dof_positions(mesh, basis)
    upwind = mesh.tri_neighbour.astype(np.int64).copy()
    shift = np.zeros((n, 3, 2))
    fb = mesh.face_bc[mesh.tri_faces]
    code = np.where(fb >= 0, bc_codes[np.clip(fb, 0, None)] if bc_codes.size else 0, 0)
    for i, il in zip(*np.nonzero((fb >= 0) & (code == BC_PERIODIC))):
        fc = mesh.tri_faces[i, il]
        upwind[i, il] = bcdata.periodic_tri[fc]
        bcp = mesh.face_bc[mesh.face_pair[fc]]
        shift[i, il] = (xoff[bcp], yoff[bcp])
    emap = np.full((n, 3, nf), -1, dtype=np.int64)
    for i in range(n):
        for il in range(3):
            if upwind[i, il] < 0:
                continue
            theirs = pos[upwind[i, il]] + shift[i, il]
            for b in range(nf):
                emap[i, il, b] = np.linalg.norm(theirs - pos[i, edofs[il][b]], axis=-1).argmin()
    return upwind.astype(np.int32), emap.astype(np.int32)


@pytest.mark.parametrize("deg", [1, 2, 3, 4])
@pytest.mark.parametrize("kind", ["cavity:6", "cavity:5:smootherstep", "periodic"])
def test_edge_maps_match_brute_force(deg, kind):
    from cases import periodic_case, small_case
    case = periodic_case(deg, 4, 8, 1.0, 0.1, mesh="channel:6") if kind == "periodic" else \
        small_case(deg, 4, 8, 1.0, 0.1, mesh=kind)
    disc = Discretisation.build(case)
    xoff = np.asarray([b.xoff for b in case.boundaries], dtype=float)
    yoff = np.asarray([b.yoff for b in case.boundaries], dtype=float)
    up, em = _edge_maps_brute_force(disc.mesh, disc.basis, disc.edge_dofs, disc.bcdata,
                                    np.asarray(case.bc_codes()), xoff, yoff)
    assert np.array_equal(disc.upwind_tri, up)
    assert np.array_equal(disc.edge_map, em)
