"""The GSIS trace solve on the device (nested-dissection multifrontal
factors, ``pbte_nd_forward`` / ``pbte_nd_backward``) against scipy's sparse
LU, and complete GSIS solves with it against the host SuperLU solve that
pybte uses: same iteration counts, fields within 1e-12."""
import numpy as np
import pytest
import torch
from scipy.sparse.linalg import spsolve

from cases import case_from_meta, periodic_case, small_case
from pbte_gb300 import Solver
from pbte_gb300.discretisation import Discretisation
from pbte_gb300.trace_nd import NestedDissectionSolver
from test_trace_nd import trace_pattern_matrix

pytestmark = pytest.mark.gpu


def _rel(a, b):
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))


@pytest.mark.parametrize("periodic", [False, True])
@pytest.mark.parametrize("b", [6, 9, 12])
def test_device_trace_solve_matches_sparse_lu(cuda, periodic, b):
    case = periodic_case(1, 4, 8, 1.0, 0.1, mesh="channel:12") if periodic else small_case(1, 4, 8, 1.0, 0.1,
                                                                                            mesh="cavity:12")
    mesh = Discretisation.build(case).mesh
    K = trace_pattern_matrix(mesh, b, seed=b, periodic=periodic)
    s = NestedDissectionSolver(K, mesh.nodes[mesh.face_nodes].mean(axis=1), b, device=cuda, leaf=16)
    assert s.check_residual < 1e-13
    rhs = np.random.default_rng(7).standard_normal(K.shape[0])
    x = s.solve(torch.from_numpy(rhs).to(cuda))
    x2 = s.solve(torch.from_numpy(rhs).to(cuda))
    assert torch.equal(x, x2)                      # deterministic
    ref = spsolve(K.tocsc(), rhs)
    assert _rel(x.cpu().numpy(), ref) < 1e-11


@pytest.mark.parametrize("kind", ["adiabatic", "isothermal", "periodic", "deg3"])
def test_gsis_step_matches_oracle(cuda, kind):
    """One GSIS correction (hot source, trace right-hand side with the wall
    traces, trace solve, local recovery, damped correction) from the same
    seeded distribution, GPU against the oracle."""
    from oracle.oracle import GSIS as OracleGSIS
    from oracle.oracle import Oracle
    if kind == "periodic":
        case = periodic_case(2, 4, 8, 0.05, 0.005, accflag=1)
    elif kind == "deg3":
        case = small_case(3, 4, 8, 0.05, 0.005, accflag=1)
    else:
        case = small_case(2 if kind == "adiabatic" else 1, 4, 8, 0.05, 0.005, accflag=1,
                          south="nonthermalising" if kind == "adiabatic" else "thermalising")
    s = Solver(case)
    o = Oracle(s.disc, nthreads=4)
    og = OracleGSIS(o)
    rng = np.random.default_rng(31)
    o.vdf[:] = rng.standard_normal(o.vdf.shape)
    s.vdf.copy_(torch.from_numpy(o.vdf))
    og.apply()
    s.acc.apply()
    torch.cuda.synchronize()
    assert _rel(s.acc.uq.cpu().numpy(), og.uq) < 1e-10
    assert _rel(s.vdf.cpu().numpy(), o.vdf) < 1e-10
    h = s.mom.host()
    for k in ("ts", "qxs", "qys", "temp"):
        assert _rel(h[k], getattr(o, k)) < 1e-10, k


@pytest.mark.parametrize("name", ["precond_diffusive", "precond_ballistic"])
def test_krylov_moment_preconditioner_matches_reference(cuda, name):
    """GMRES(30) with pybte's moment preconditioner (scheme.krylov_precond)
    against pybte's own run: sweeps within 2 %, temperatures within 1e-8."""
    from cases import golden, meta
    m = meta()[name]
    z = golden("krylov_precond")
    c = small_case(1, 4, 8, m["tau_r"], 0.1 * m["tau_r"], south="thermalising", accflag=1, method="krylov",
                   krylov_restart=30)
    c.scheme.krylov_precond = True
    rec = Solver(c).run()
    assert rec.converged == m["converged"]
    assert rec.diagnostics["krylov_precond"] is True
    assert abs(rec.iterations - m["iterations"]) <= max(2, int(0.02 * m["iterations"]))
    assert _rel(rec.temp, z[f"{name}_temp"]) < 1e-8


@pytest.mark.parametrize("name", ["gsis_deg2_adiabatic", "gsis_deg1_isothermal"])
def test_gsis_device_and_host_trace_solves_agree(cuda, name):
    recs = {}
    for where in ("host", "device"):
        c = case_from_meta(name)
        c.performance.trace_solver = where
        recs[where] = Solver(c).run()
    a, d = recs["host"], recs["device"]
    assert a.converged and d.converged and a.iterations == d.iterations
    assert _rel(d.temp, a.temp) < 1e-12 and _rel(d.temp_dofs, a.temp_dofs) < 1e-12
    assert _rel(d.qx_dofs, a.qx_dofs) < 1e-11
