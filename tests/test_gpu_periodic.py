"""Periodic faces on the GPU, through the C ABI, against the oracle and the
reference's periodic fixtures (tests/golden/periodic.npz).

pybte's source-iteration sweep reads a periodic partner's *current* values:
this sweep's when the partner comes first in the direction's TRI_ORDER,
the previous sweep's otherwise.  The GPU schedule makes the first kind a
dependency and reads the second from a snapshot taken before the sweep; the
Krylov path reads every partner from pbuf (its explicit state).
Tolerances as for the other FP64 kernels: 1e-11 per sweep, complete solves
1e-10 (GMRES 1e-8).
"""
import numpy as np
import pytest
import torch

from cases import golden, meta, periodic_case, task_case
from oracle.oracle import Oracle
from pbte_gb300 import Solver, _lib
from pbte_gb300.config import Case
from pbte_gb300.output import locate_points, sample_fields

pytestmark = pytest.mark.gpu


def _rel(a, b):
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))


def _seed(s, o, seed):
    rng = np.random.default_rng(seed)
    for k in ("ts", "qxs", "qys"):
        v = rng.standard_normal(getattr(o, k).shape) * (1.0 if k == "ts" else 0.3)
        getattr(o, k)[:] = v
        getattr(s.mom, k).copy_(torch.from_numpy(v))
    o.vdf[:] = rng.standard_normal(o.vdf.shape)
    s.vdf.copy_(torch.from_numpy(o.vdf))
    return rng


@pytest.mark.parametrize("deg", [1, 2, 3])
@pytest.mark.parametrize("mode", ["precomputed", "onthefly"])
@pytest.mark.parametrize("variant", [0, 1])
@pytest.mark.parametrize("mesh", ["channel:5:smootherstep", "channel:16"])
def test_periodic_sweeps_match_oracle(cuda, deg, mode, variant, mesh):
    """Two source-iteration sweeps in a row (the second reads lagged partners
    from the first), the transport residual, then the pbuf form.  variant 0
    is the ring sweep, 1 the level-serial one."""
    s = Solver(periodic_case(deg, 4, 8, 0.5, 0.05, sweep_mode=mode, mesh=mesh))
    assert s.ctx.mode == mode
    s.ctx.set_variant(variant)
    o = Oracle(s.disc, nthreads=4)
    rng = _seed(s, o, 40 + deg)
    for _ in range(2):
        o.sweep()
        s.ctx.sweep(s.mom, s.vdf)
        torch.cuda.synchronize()
        assert _rel(s.vdf.cpu().numpy(), o.vdf) < 1e-11
    assert s.ctx.true_residual(s.mom, s.vdf) == pytest.approx(o.true_residual(), rel=1e-9)
    pbuf = rng.standard_normal(o.pbuf.shape)
    o.pbuf[:] = pbuf
    o.use_pbuf = True
    s.ctx.pbuf.copy_(torch.from_numpy(pbuf))
    s.ctx.use_pbuf = True
    o.sweep()
    s.ctx.sweep(s.mom, s.vdf)
    s.ctx.use_pbuf = False
    torch.cuda.synchronize()
    assert _rel(s.vdf.cpu().numpy(), o.vdf) < 1e-11
    s.ctx.set_variant(0)


@pytest.mark.parametrize("deg", [1, 2])
def test_periodic_sweep_matches_reference_fixture(cuda, deg):
    z = golden("periodic")
    s = Solver(periodic_case(deg, 4, 8, 0.5, 0.05))
    for k in ("ts", "qxs", "qys"):
        getattr(s.mom, k).copy_(torch.from_numpy(z[f"deg{deg}_{k}"]))
    s.vdf.copy_(torch.from_numpy(z[f"deg{deg}_vdf_in"]))
    s.ctx.sweep(s.mom, s.vdf)
    assert _rel(s.vdf.cpu().numpy(), z[f"deg{deg}_vdf_cis"]) < 1e-11
    s.vdf.copy_(torch.from_numpy(z[f"deg{deg}_vdf_in"]))
    s.ctx.pbuf.copy_(torch.from_numpy(z[f"deg{deg}_pbuf"]))
    s.ctx.use_pbuf = True
    s.ctx.sweep(s.mom, s.vdf)
    s.ctx.use_pbuf = False
    assert _rel(s.vdf.cpu().numpy(), z[f"deg{deg}_vdf_pbuf"]) < 1e-11


def test_periodic_gather_and_scatter(cuda):
    s = Solver(periodic_case(2, 4, 8, 0.5, 0.05))
    L = _lib.lib()
    import ctypes
    n = ctypes.c_int64()
    _lib.check(L.pbte_periodic_count(s.ctx.handle, ctypes.byref(n)), "count")
    pfaces = np.flatnonzero(s.bcdata.periodic_tri >= 0)
    assert n.value == pfaces.size > 0
    vdf = torch.randn(s.vdf.shape, dtype=torch.float64, device=cuda)
    out = torch.zeros((s.ndir, n.value, s.ndof), dtype=torch.float64, device=cuda)
    _lib.check(L.pbte_periodic_gather(s.ctx.handle, vdf.data_ptr(), out.data_ptr(), None), "gather")
    v = vdf.cpu().numpy()
    assert np.array_equal(out.cpu().numpy(), v[:, s.bcdata.periodic_tri[pfaces], :])
    pbuf = torch.zeros_like(s.ctx.pbuf)
    _lib.check(L.pbte_periodic_scatter(s.ctx.handle, out.data_ptr(), pbuf.data_ptr(), None), "scatter")
    p = pbuf.cpu().numpy()
    assert np.array_equal(p[:, pfaces, :], out.cpu().numpy())
    others = np.setdiff1d(np.arange(s.mesh.n_faces), pfaces)
    assert not p[:, others, :].any()


@pytest.mark.parametrize("name", ["cis_deg1", "gsis_deg2", "krylov_deg2"])
def test_periodic_solves_match_reference(cuda, name):
    z = golden("periodic")
    m = meta()[f"periodic_{name}"]
    kw = {k: m[k] for k in ("deg", "npole", "nazim", "tau_r", "tau_n")}
    krylov = m.get("method") == "krylov"
    s = Solver(periodic_case(**kw, accflag=m.get("accflag", 0), method=m.get("method", "source"),
                             krylov_restart=30 if krylov else None))
    rec = s.run()
    assert rec.converged
    if krylov:
        assert abs(rec.iterations - m["iterations"]) <= max(1, int(0.02 * m["iterations"]))
        assert _rel(rec.temp, z[f"{name}_temp"]) < 1e-8
    else:
        assert abs(rec.iterations - m["iterations"]) <= (0 if m.get("accflag", 0) == 0 else 1)
        assert _rel(rec.temp, z[f"{name}_temp"]) < 1e-10
        assert _rel(rec.temp_dofs, z[f"{name}_ts"]) < 1e-10


def test_f3_task_certified_solution(cuda):
    z = golden("periodic")
    rec = Solver(task_case("F3", "1_1")).run()
    assert rec.converged
    assert abs(rec.iterations - meta()["task_F3_1_1"]["iterations"]) <= 1
    assert _rel(rec.temp, z["task_F3_1_1__temp"]) < 1e-9


def test_periodic_reproduces_a_one_dimensional_solution(cuda):
    """pybte's cases/channel_periodic_gsis.yaml (walls in y, a periodic pair
    in x, DEG 3, 20 x 40 ordinates, tau_R = 1e-2, GSIS) and the checks of
    its tests/integration/test_deviations.py:67-87: the answer does not
    depend on x, and int T dA = 1/2."""
    c = Case.from_dict({
        "iteration": {"tol": 1e-8, "tmax": 200000}, "scheme": {"accflag": 1},
        "velmesh": {"npole": 20, "nazim": 40}, "dg": {"deg": 3},
        "flow": {"cv": 1.0, "vg": 1.0, "tau_r": 1e-2, "tau_n": 1e5, "tau_thr": 1.0},
        "mesh": {"file": "channel:10:smootherstep"},
        "boundaries": [{"name": "Swall", "phyid": 11, "type": "thermalising", "temp": 0.0},
                       {"name": "NWall", "phyid": 12, "type": "thermalising", "temp": 1.0},
                       {"name": "Master", "phyid": 13, "type": "periodic", "temp": 0.0, "xoff": -1.0},
                       {"name": "Slave", "phyid": 14, "type": "periodic", "temp": 0.0, "xoff": 1.0}]})
    s = Solver(c)
    rec = s.run()
    assert rec.converged
    assert int(s.bcdata.periodic_flip.sum()) > 0
    px = np.linspace(0.02, 0.98, 21)
    py = np.linspace(0.05, 0.95, 19)
    tri = locate_points(s.mesh, px, py)
    cx, cy, dw = s.vel.flat()
    T, qx, qy, *_ = sample_fields(s.mesh, s.disc.basis, s.vdf, cx, cy, dw, 1.0, px, py, tri)
    assert np.ptp(T, axis=0).max() < 1e-3 * np.ptp(T)
    assert np.abs(qx).max() < 1e-3 * np.abs(qy).mean()
    assert rec.mass == pytest.approx(0.5, abs=1e-5)


def test_mixed_precision_refuses_periodic_faces(cuda):
    with pytest.raises(NotImplementedError, match="periodic"):
        Solver(periodic_case(1, 4, 8, 1.0, 0.1, precision="mixed")).run()
