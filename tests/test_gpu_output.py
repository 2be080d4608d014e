"""GPU field output, restart files and run-record plumbing, through the C ABI,
against the reference's outputs.

* ``locate_points``: bit-exact element ids (the kernel evaluates pybte's
  sub-areas in its operation order, without FMA contraction).
* ``sample_fields`` on the reference's own distribution and GSIS unknowns:
  1e-12 of each field's largest value (the moment sums and basis
  evaluation run in a different order than numpy's einsums).
* Fields of a complete GPU solve: 1e-9 against the reference solve's.
* The reference's frozen 109 x 109 field values of its cavity case
  (``tests/integration/test_regression.py:99-125`` of pybte): rel 1e-9, as
  there.
* Restart contract (``tests/unit/test_config.py:130-185`` of pybte):
  round trip, stale file, size mismatch.
"""
import json

import numpy as np
import pytest
import torch

from cases import golden, meta, small_case
from pbte_gb300 import Solver
from pbte_gb300.config import Case
from pbte_gb300.output import locate_points, sample_fields, sampling_grid

pytestmark = pytest.mark.gpu


def _rel(a, b):
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))


@pytest.fixture(scope="module")
def z():
    return golden("field_output")


def _case(**over):
    m = meta()["field_output"]
    kw = dict(deg=m["deg"], npole=m["npole"], nazim=m["nazim"], tau_r=m["tau_r"], tau_n=m["tau_n"],
              accflag=m["accflag"])
    kw.update(over)
    return small_case(**kw)


def test_locate_points_bitwise(cuda, z):
    s = Solver(_case(accflag=0))
    assert np.array_equal(locate_points(s.mesh, z["px"], z["py"]), z["triid"])
    assert np.array_equal(locate_points(s.mesh, z["pxo"], z["pyo"]), z["triido"])
    nan = locate_points(s.mesh, np.array([np.nan, 0.5]), np.array([0.5]))
    assert nan[0, 0] == -1 and nan[1, 0] >= 0


def test_sample_fields_of_the_reference_state(cuda, z):
    s = Solver(_case(accflag=0))
    cx, cy, dw = s.vel.flat()
    got = sample_fields(s.mesh, s.disc.basis, z["vdf"], cx, cy, dw, 1.0, z["px"], z["py"], z["triid"],
                        uq=z["uq"])
    for k, g in zip(("T", "qx", "qy", "Nxx", "Nxy", "Nyy"), got):
        assert _rel(g, z[k]) < 1e-12, k
    # device-resident inputs give the same answer
    dv = torch.from_numpy(z["vdf"]).to(cuda)
    du = torch.from_numpy(z["uq"]).to(cuda)
    again = sample_fields(s.mesh, s.disc.basis, dv, cx, cy, dw, 1.0, z["px"], z["py"], z["triid"], uq=du)
    for a, b in zip(got, again):
        assert np.array_equal(a, b)
    To, qxo, qyo, nxx, nxy, nyy = sample_fields(s.mesh, s.disc.basis, z["vdf"], cx, cy, dw, 2.0, z["pxo"],
                                                z["pyo"], z["triido"])
    assert _rel(To, z["To"]) < 1e-12 and _rel(qxo, z["qxo"]) < 1e-12 and _rel(qyo, z["qyo"]) < 1e-12
    assert not (nxx.any() or nxy.any() or nyy.any())
    outside = z["triido"] < 0
    assert outside.any() and not To[outside].any()


def test_fields_of_a_gpu_gsis_solve(cuda, z, tmp_path):
    c = _case()
    c.basedir = str(tmp_path)
    c.output.dir = str(tmp_path / "out")
    c.output.tecplot = True
    s = Solver(c)
    rec = s.run()
    assert rec.converged and abs(rec.iterations - meta()["field_output"]["iterations"]) <= 1
    written = s.write_outputs(rec)
    f = np.load(written["field_npz"])
    assert np.array_equal(f["triid"], z["triid"])
    for k in ("T", "qx", "qy", "Nxx", "Nxy", "Nyy"):
        assert _rel(f[k], z[k]) < 1e-9, k
    d = json.loads((tmp_path / "out" / "run_record.json").read_text())
    assert set(z["record_keys"]) <= set(d)
    assert d["scheme"] == "GSIS" and len(d["config_hash"]) == 64 and d["environment"]["numpy"]
    assert d["diagnostics"]["global_solve_count"] == rec.iterations
    line = (tmp_path / "out" / "RunTime.txt").read_text().splitlines()[-1]
    assert line.split()[:4] == ["GSIS", "1.00E-01", "1.00E-02", "50"]
    assert (tmp_path / "out" / "field.dat").read_text().startswith(' VARIABLES="x","y","T"')


def test_reference_frozen_field_values(cuda):
    """pybte's cavity case (its meshes/A1_Nx11_Ny11.msh is the 10 x 10
    smootherstep cavity) at tau_R = 0.1, DEG 3, 20 x 40 ordinates, CIS."""
    c = Case.from_dict({
        "iteration": {"tol": 1e-8, "tmax": 8000000}, "scheme": {"accflag": 0},
        "velmesh": {"npole": 20, "nazim": 40}, "dg": {"deg": 3},
        "flow": {"cv": 1.0, "vg": 1.0, "tau_r": 0.1, "tau_n": 1e5, "tau_thr": 1.0},
        "mesh": {"file": "cavity:10:smootherstep"},
        "boundaries": [{"name": "SWall", "phyid": 11, "type": "thermalising", "temp": 0.0},
                       {"name": "NWall", "phyid": 12, "type": "thermalising", "temp": 1.0},
                       {"name": "EWall", "phyid": 13, "type": "thermalising", "temp": 0.0},
                       {"name": "WWall", "phyid": 14, "type": "thermalising", "temp": 0.0}]})
    s = Solver(c)
    assert s.run().converged
    px, py = sampling_grid()
    tri = locate_points(s.mesh, px, py)
    assert not np.any(tri < 0)
    cx, cy, dw = s.vel.flat()
    T, qx, qy, *_ = sample_fields(s.mesh, s.disc.basis, s.vdf, cx, cy, dw, c.flow.cv, px, py, tri)
    assert T[0, 0] == pytest.approx(0.0032735050690818894, rel=1e-9)
    assert T[54, 54] == pytest.approx(0.2499447278527214, rel=1e-9)
    assert T[54, 104] == pytest.approx(0.8728271107454624, rel=1e-9)
    assert float(T.min()) == pytest.approx(0.0032735050690818894, rel=1e-9)
    assert float(T.max()) == pytest.approx(0.8983932311211115, rel=1e-9)
    assert float(np.abs(qx).max()) == pytest.approx(0.1883719557037961, rel=1e-9)
    assert float(T.mean()) == pytest.approx(0.24989294601937023, rel=1e-9)


def _tiny(tmp_path, **restart):
    c = small_case(1, 4, 4, 1e-3, 1e5, south="thermalising", tmax=2)
    c.basedir = str(tmp_path)
    c.output.dir = str(tmp_path / "out")
    for k, v in restart.items():
        setattr(c.restart, k, v)
    return c


def test_restart_roundtrip_and_name(cuda, tmp_path, z):
    s = Solver(_tiny(tmp_path))
    s.run()
    vdf = s.vdf.cpu().numpy().copy()
    path = s.save_restart()
    assert path.name == "VDFP1T50NP4NA4.out"
    s2 = Solver(_tiny(tmp_path, enabled=True, path=str(path)))
    assert np.array_equal(s2.vdf.cpu().numpy(), vdf)
    assert s2.restart_info["enabled"] is True and len(s2.restart_info["sha256"]) == 64
    np.testing.assert_array_equal(s2.vdf_fortran(), np.transpose(vdf.reshape(4, 4, 50, 3), (3, 2, 1, 0)))
    # the reference's own restart file loads into the same array
    m = meta()["field_output"]
    ref = tmp_path / m["restart_name"]
    ref.write_bytes(z["restart"].tobytes())
    c3 = _case(accflag=0)
    c3.basedir = str(tmp_path)
    c3.restart.enabled = True
    s3 = Solver(c3)
    assert np.array_equal(s3.vdf.cpu().numpy(), z["vdf"])
    assert Solver(c3).save_restart(tmp_path / "again.out").read_bytes() == z["restart"].tobytes()


def test_stale_restart_file_is_an_error(cuda, tmp_path):
    s = Solver(_tiny(tmp_path))
    assert s.save_restart().exists()
    with pytest.raises(FileExistsError, match="restart file"):
        Solver(_tiny(tmp_path))
    Solver(_tiny(tmp_path, error_on_stale=False))


def test_restart_size_mismatch_is_caught(cuda, tmp_path):
    bad = tmp_path / "junk.out"
    bad.write_bytes(b"\x00" * 64)
    with pytest.raises(ValueError, match="expected"):
        Solver(_tiny(tmp_path, enabled=True, path=str(bad)))
    with pytest.raises(FileNotFoundError):
        Solver(_tiny(tmp_path, enabled=True, path=str(tmp_path / "absent.out")))


def test_restarted_cis_matches_the_reference(cuda, tmp_path, z):
    """CIS restarted from the reference's restart file: pybte keeps its
    moments at zero and takes the wall emission from the loaded
    distribution, so the run is its own (3350 steps here); same steps and
    temperatures as the reference's restarted run."""
    m = meta()["field_output"]
    path = tmp_path / "restart.out"
    path.write_bytes(z["restart"].tobytes())
    c = _case(accflag=0)
    c.basedir = str(tmp_path)
    c.restart.enabled = True
    c.restart.path = str(path)
    rec = Solver(c).run()
    assert rec.converged and abs(rec.iterations - m["restart_cis_iterations"]) <= 1
    assert _rel(rec.temp, z["restart_cis_temp"]) < 1e-9
    n = min(rec.iterations, z["restart_cis_residuals"].size) - 1
    np.testing.assert_allclose(rec.residual_history[:n], z["restart_cis_residuals"][:n], rtol=1e-6)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_krylov_restart_starts_from_the_loaded_state(cuda, tmp_path, precision):
    """GMRES restarted from its own converged distribution starts at the
    loaded state (``pybte/krylov.py:311``) and finishes in a few sweeps."""
    def make():
        c = small_case(2, 4, 8, 0.3, 0.03, method="krylov", tol=1e-9, precision=precision)
        c.basedir = str(tmp_path)
        return c

    s = Solver(make())
    first = s.run()
    path = s.save_restart(tmp_path / "state.out")
    c2 = make()
    c2.restart.enabled = True
    c2.restart.path = str(path)
    again = Solver(c2).run()
    assert again.converged
    assert again.iterations < max(6, first.iterations // 4), (again.iterations, first.iterations)
    assert _rel(again.temp, first.temp) < 1e-7


def test_callback_and_true_residual_follow_the_graph_path(cuda):
    """CIS with a callback (host-driven loop) takes the graph-captured run's
    iterations and residuals; the true residual is recorded on request."""
    c = small_case(1, 4, 8, 1.0, 0.1)
    base = Solver(c).run()
    seen = []
    c2 = small_case(1, 4, 8, 1.0, 0.1)
    c2.iteration.true_residual = True
    c2.iteration.true_residual_every = 5
    rec = Solver(c2).run(callback=lambda step, res, solver: seen.append((step, res)))
    assert rec.iterations == base.iterations
    assert [s for s, _ in seen] == list(range(1, rec.iterations + 1))
    np.testing.assert_allclose([r for _, r in seen], base.residual_history, rtol=1e-9)
    assert rec.residual_true.shape == (rec.iterations,)
    assert np.isfinite(rec.residual_true[4]) and np.isnan(rec.residual_true[3])
