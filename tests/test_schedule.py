"""Direction classes as the context schedules them (pbte_direction_classes,
host only) against the face-by-face sign patterns formed here with numpy, on
meshes whose face normals take a few values (structured squares) and many
(graded squares, a periodic channel)."""
import numpy as np
import pytest

from cases import periodic_case, small_case
from pbte_gb300 import _lib
from pbte_gb300.discretisation import Discretisation
from pbte_gb300.sweep import direction_classes


def numpy_classes(disc):
    """Sign of c.n on every interior and periodic face (from the face's first
    side), grouped by first appearance."""
    m, bd = disc.mesh, disc.bcdata
    cx, cy, _ = disc.vel.flat()
    fb = np.asarray(m.face_bc)
    bc_type = np.asarray(bd.bc_type)
    include = (fb < 0) | ((fb >= 0) & (bc_type[np.maximum(fb, 0)] == 3))
    ft, fl = np.asarray(m.face_tri), np.asarray(m.face_lfc)
    side = np.where(ft[:, 0] >= 0, 0, 1)
    rows = np.arange(ft.shape[0])
    t, lf = ft[rows, side][include], fl[rows, side][include]
    nx, ny = m.tri_normal[t, lf, 0], m.tri_normal[t, lf, 1]
    pat = np.sign(np.outer(cx, nx) + np.outer(cy, ny)).astype(np.int8)
    seen, out = {}, np.empty(cx.size, dtype=np.int32)
    for d in range(cx.size):
        out[d] = seen.setdefault(pat[d].tobytes(), len(seen))
    return out


@pytest.mark.parametrize("mesh", ["cavity:12", "cavity:5:smootherstep", "cavity:10:smootherstep", "channel:9"])
@pytest.mark.parametrize("ang", [(4, 8), (8, 32)])
def test_direction_classes_match_face_by_face_patterns(mesh, ang):
    try:
        _lib.lib()
    except RuntimeError as e:
        pytest.skip(f"library unavailable: {e}")
    disc = Discretisation.build(small_case(1, *ang, 1.0, 0.1, mesh=mesh))
    got = direction_classes(disc)
    assert np.array_equal(got, numpy_classes(disc))
    assert got.max() + 1 == len(set(got.tolist()))


def test_direction_classes_with_periodic_faces():
    try:
        _lib.lib()
    except RuntimeError as e:
        pytest.skip(f"library unavailable: {e}")
    disc = Discretisation.build(periodic_case(1, 8, 32, 1.0, 0.1, mesh="channel:12"))
    assert np.array_equal(direction_classes(disc), numpy_classes(disc))


def numpy_levels(disc, d, order):
    """Wavefront levels restated: walking pybte's TRI_ORDER for ordinate d,
    an element sits one level past the deepest element it waits for: an
    interior upwind neighbour, or a periodic partner earlier in that order."""
    m, bd = disc.mesh, disc.bcdata
    cx, cy, _ = disc.vel.flat()
    up = np.asarray(disc.upwind_tri)
    fb = np.asarray(m.face_bc)
    bc_type = np.asarray(bd.bc_type)
    pos = np.empty(m.n_tris, dtype=np.int64)
    pos[order] = np.arange(m.n_tris)
    s = cx[d] * m.tri_normal[:, :, 0] + cy[d] * m.tri_normal[:, :, 1]
    level = np.zeros(m.n_tris, dtype=np.int64)
    for i in order:
        for il in range(3):
            nb, f = up[i, il], m.tri_faces[i, il]
            if nb < 0 or not s[i, il] < 0.0:
                continue
            if fb[f] >= 0 and not (bc_type[fb[f]] == 3 and pos[nb] < pos[i]):
                continue
            level[i] = max(level[i], level[nb] + 1)
    return level


@pytest.mark.parametrize("kind", ["cavity:12", "cavity:10:smootherstep", "periodic"])
def test_direction_levels_match_order_walk(kind):
    try:
        _lib.lib()
    except RuntimeError as e:
        pytest.skip(f"library unavailable: {e}")
    from oracle.oracle import reference_order
    from pbte_gb300.sweep import direction_levels
    case = periodic_case(1, 4, 8, 1.0, 0.1, mesh="channel:12") if kind == "periodic" else \
        small_case(1, 4, 8, 1.0, 0.1, mesh=kind)
    disc = Discretisation.build(case)
    order, _ = reference_order(disc)
    for d in range(order.shape[0]):
        got = direction_levels(disc, d)
        assert np.array_equal(got, numpy_levels(disc, d, order[d])), d


def test_host_schedule_entries_reject_bad_arguments():
    import ctypes

    try:
        L = _lib.lib()
    except RuntimeError as e:
        pytest.skip(f"library unavailable: {e}")
    from pbte_gb300.sweep import case_desc
    disc = Discretisation.build(small_case(1, 4, 8, 1.0, 0.1, mesh="cavity:4"))
    desc, keep = case_desc(disc)
    n = ctypes.c_int32()
    cls = np.zeros(disc.vel.flat()[0].size, dtype=np.int32)
    lev = np.zeros(disc.mesh.n_tris, dtype=np.int32)
    assert L.pbte_direction_classes(None, cls.ctypes.data, ctypes.byref(n)) == -1
    assert L.pbte_direction_classes(ctypes.byref(desc), None, ctypes.byref(n)) == -1
    assert L.pbte_direction_levels(ctypes.byref(desc), -1, lev.ctypes.data, ctypes.byref(n)) == -1
    assert L.pbte_direction_levels(ctypes.byref(desc), cls.size, lev.ctypes.data, ctypes.byref(n)) == -1
    assert L.pbte_direction_levels(ctypes.byref(desc), 0, lev.ctypes.data, ctypes.byref(n)) == 0
    assert n.value == lev.max() + 1
    bad = np.array(keep["face_bc"])
    bad[0] = 1000                                  # a boundary condition index past nbc
    desc.face_bc = bad.ctypes.data_as(ctypes.POINTER(ctypes.c_int32))
    assert L.pbte_direction_classes(ctypes.byref(desc), cls.ctypes.data, ctypes.byref(n)) == -1
