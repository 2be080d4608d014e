"""Host side of field output, restart files and run records, against the
reference's own outputs (tests/golden/field_output.npz, written by
make_golden.py from pybte's io_output and driver): the sampling grid, the
point bins' candidate lists, the Tecplot and RunTime.txt bytes, the restart
byte layout, the run-record helpers, and the shipped mesh."""
import ctypes
import json

import numpy as np
import pytest

from cases import golden, meta, small_case
from pbte_gb300 import _lib
from pbte_gb300.discretisation import Discretisation
from pbte_gb300.mesh import structured_square
from pbte_gb300.output import PointBins, append_runtime_log, sampling_grid, write_tecplot
from pbte_gb300.solver import RunRecord


@pytest.fixture(scope="module")
def z():
    return golden("field_output")


@pytest.fixture(scope="module")
def mesh():
    m = meta()["field_output"]
    case = small_case(m["deg"], m["npole"], m["nazim"], m["tau_r"], m["tau_n"], accflag=m["accflag"])
    return Discretisation.build(case).mesh


def test_sampling_grid_is_bitwise_the_reference(z):
    px, py = sampling_grid()
    assert px.tobytes() == z["px"].tobytes() and py.tobytes() == z["py"].tobytes()
    qx, qy = sampling_grid(7, 5)
    assert np.array_equal(qx, np.linspace(0, 1, 7)) and np.array_equal(qy, np.linspace(0, 1, 5))


def _scan(tx, ty, px, py, candidates):
    """The sub-area test in pybte's operation order over each point's
    candidate list, first pass wins (a host restatement of the kernel)."""
    out = np.full((px.size, py.size), -1, dtype=np.int32)
    for i, x in enumerate(px):
        for j, y in enumerate(py):
            for k in candidates(x, y):
                ok = True
                for il in range(3):
                    i2 = (il + 1) % 3
                    a = 0.5 * (x * (ty[k, il] - ty[k, i2]) - y * (tx[k, il] - tx[k, i2])
                               + (tx[k, il] * ty[k, i2] - tx[k, i2] * ty[k, il]))
                    ok &= bool(a >= -1e-12)
                if ok:
                    out[i, j] = k
                    break
    return out


@pytest.mark.parametrize("grid", ["sampling", "outside"])
def test_point_bins_give_the_first_match(z, mesh, grid):
    tx, ty = mesh.nodes[mesh.tri_nodes, 0], mesh.nodes[mesh.tri_nodes, 1]
    px, py, want = (z["px"], z["py"], z["triid"]) if grid == "sampling" else (z["pxo"], z["pyo"], z["triido"])
    for per_side in (None, 1, 3, 16):
        b = PointBins(tx, ty, per_side)
        assert b.start[-1] == b.items.size
        for cell in range(b.nbx * b.nby):                # each bin lists elements in increasing order
            assert np.all(np.diff(b.items[b.start[cell]:b.start[cell + 1]]) > 0)

        def cands(x, y, b=b):
            c = int(b.cell_of(np.array([x]), np.array([y]))[0])
            return b.items[b.start[c]:b.start[c + 1]]

        assert np.array_equal(_scan(tx, ty, px, py, cands), want), per_side


def test_point_bins_cover_every_accepted_element(mesh):
    """Points on and just past every element edge and corner: whatever the
    full scan accepts must be among the point's bin candidates."""
    tx, ty = mesh.nodes[mesh.tri_nodes, 0], mesh.nodes[mesh.tri_nodes, 1]
    b = PointBins(tx, ty, 12)
    rng = np.random.default_rng(5)
    for k in range(mesh.n_tris):
        for il in range(3):
            i2 = (il + 1) % 3
            for t in (0.0, 1.0, rng.random()):
                x = tx[k, il] + t * (tx[k, i2] - tx[k, il])
                y = ty[k, il] + t * (ty[k, i2] - ty[k, il])
                for dx, dy in ((0, 0), (1e-13, 0), (0, -1e-13), (-1e-13, 1e-13)):
                    px, py = np.array([x + dx]), np.array([y + dy])
                    full = _scan(tx, ty, px, py, lambda *_: range(mesh.n_tris))
                    c = int(b.cell_of(px, py)[0])
                    if full[0, 0] >= 0:
                        assert full[0, 0] in b.items[b.start[c]:b.start[c + 1]]


def test_tecplot_and_runtime_log_bytes(z, tmp_path):
    p = write_tecplot(tmp_path / "f.dat", z["pxo"], z["pyo"], [z["To"], z["qxo"], z["qyo"]], ["T", "qx", "qy"])
    assert p.read_bytes() == z["tecplot"].tobytes()
    log = tmp_path / "RunTime.txt"
    for args in (("CIS", 1e-3, 1e5, 200, 20, 40, 183211, 48123.46),
                 ("GSIS", 0.1, 0.01, 50, 4, 8, 17, 0.05),
                 ("KRYLOV", 2.5e-7, 3e12, 20000, 10, 20, 9, 123456789.0)):
        append_runtime_log(log, *args)
    assert log.read_bytes() == z["runtime_log"].tobytes()


def test_restart_bytes_are_the_c_order_distribution(z):
    """The Fortran VDF(NDOF, N_TRIS, NPOLE, NAZIM) file holds exactly the
    bytes of the C-order (ndir, n_tris, ndof) array."""
    assert z["vdf"].astype("<f8").tobytes() == z["restart"].tobytes()
    m = meta()["field_output"]
    nd = (m["deg"] + 1) * (m["deg"] + 2) // 2
    f = z["restart"].view("<f8").reshape((nd, 50, m["npole"], m["nazim"]), order="F")
    back = np.transpose(f, (3, 2, 1, 0)).reshape(z["vdf"].shape)
    assert np.array_equal(back, z["vdf"])


def test_run_record_helpers_match_the_reference(z, tmp_path):
    m = meta()["field_output"]
    rec = RunRecord(iterations=m["iterations"], residual_history=z["residuals"], temp=np.ones(3),
                    temp_dofs=np.zeros((6, 3)))
    assert rec.final_residual == m["final_residual"]
    assert rec.contraction == pytest.approx(m["contraction"], rel=1e-15)
    assert rec.error_estimate == pytest.approx(m["error_estimate"], rel=1e-14)
    d = rec.to_dict(include_fields=False)
    assert set(z["record_keys"]) <= set(d)
    assert d["temp_dofs"] is None and d["temp"] == [1.0, 1.0, 1.0]
    back = json.loads(rec.to_json(tmp_path / "r.json").read_text())
    assert back["contraction"] == pytest.approx(m["contraction"])
    npz = np.load(rec.to_npz(tmp_path / "r.npz"))
    assert np.array_equal(npz["residual_history"], z["residuals"])
    assert json.loads(str(npz["meta"]))["iterations"] == m["iterations"]
    short = RunRecord(residual_history=np.array([1.0, 0.5, 0.25]))
    assert np.isnan(short.contraction) and np.isnan(short.error_estimate)
    rising = RunRecord(residual_history=np.linspace(1.0, 2.0, 12))
    assert np.isnan(rising.contraction)


def test_shipped_mesh_is_the_structured_generator(z):
    """pybte's meshes/A1_Nx11_Ny11.msh (the reference cavity case) is the
    10 x 10 smootherstep cavity: identical nodes, triangles and wall lines."""
    raw = structured_square(10, "cavity", "smootherstep")
    assert np.array_equal(raw.nodes, z["shipped_nodes"])
    assert np.array_equal(raw.tri_nodes, z["shipped_tri_nodes"])
    assert np.array_equal(raw.line_nodes, z["shipped_line_nodes"])
    assert np.array_equal(raw.line_phyid, z["shipped_line_phyid"])


def test_output_entry_points_reject_bad_sizes_on_the_host():
    """Bad sizes come back as PBTE_ERR_ARG before any launch (no GPU here)."""
    try:
        _lib.build()
    except (OSError, RuntimeError) as e:                 # no nvcc in this environment
        if not _lib.LIB_PATH.exists():
            pytest.skip(f"library not built and cannot build here: {e}")
    L = _lib.lib()
    buf = (ctypes.c_double * 16)()
    p = ctypes.cast(buf, ctypes.c_void_p)
    assert L.pbte_field_moments(p, 0, 4, 3, p, p, p, p, p, p, None) == -1
    assert L.pbte_locate_points(p, p, 4, 0.0, 0.0, 0.0, 1.0, 1, 1, p, p, p, 2, p, 2, p, None) == -1
    assert L.pbte_locate_points(p, p, 4, 0.0, 0.0, 1.0, 1.0, 1, 1, p, p, p, 0, p, 2, p, None) == -1
    assert L.pbte_sample_fields(p, p, p, p, 2, p, 2, p, p, 16, p, p, p, 4, 1.0, None, p, None) == -1
    assert L.pbte_sample_fields(p, p, p, p, 2, p, 2, p, p, 3, p, p, p, 4, 1.0, None, None, None) == -1
