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
