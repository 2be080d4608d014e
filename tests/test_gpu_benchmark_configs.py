"""The benchmark's own configurations, solved on the GPU and compared with
the reference.

* 800-triangle square (uniform 20 x 20 grid, P1, 64 ordinates = npole 4 x
  nazim 16, Kn_R = 1, Kn_N = 0.1, CIS to 1e-8): against pybte itself
  (``tests/golden/c1_square20_cis.npz``, made by ``make_golden.py --c1-only``
  from pybte's ``Solver(case).run()``): the same 108 iterations, fields within
  1e-10.
* 8192-triangle square (uniform 64 x 64, P2, 256 ordinates = 8 x 32,
  Kn_N = 0.1 Kn_R): against the oracle (``tests/golden/c2_square64_oracle``,
  made by ``make_c2_fixtures.py``; the oracle is pinned to pybte by the other
  fixtures).  FP64 GMRES(30) at Kn_R = 10, 1, 0.1, CIS at 10 and GSIS at 0.01:
  sweep counts within one and relative L2 <= 1e-10 on temperature and heat
  flux.  The mixed FP32/FP64 solve at every Kn_R: relative L2 <= 1e-8 against
  the oracle's fixed point (its GMRES to 1e-12).
"""
import json

import numpy as np
import pytest

from cases import GOLDEN, golden
from pbte_gb300 import Solver, square_case

pytestmark = pytest.mark.gpu

C2 = (64, 2, 8, 32)


def rel_l2(a, b) -> float:
    a, b = np.asarray(a, dtype=float), np.asarray(b, dtype=float)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def c2_fixture():
    z = np.load(GOLDEN / "c2_square64_oracle.npz")
    return z, json.loads((GOLDEN / "c2_square64_oracle.json").read_text())


def test_c1_square20_cis_matches_pybte(cuda):
    z = golden("c1_square20_cis")
    rec = Solver(square_case(20, 1, 4, 16, tau_r=1.0, tau_n=0.1, tol=1e-8, tmax=5000)).run()
    assert rec.converged
    assert rec.iterations == int(z["iterations"]) == 108
    for got, want in ((rec.temp, z["temp"]), (rec.qx, z["qx"]), (rec.qy, z["qy"]), (rec.temp_dofs, z["ts"]),
                      (rec.qx_dofs, z["qxs"])):
        assert rel_l2(got, want) <= 1e-10
    assert float(np.sum(rec.qx)) == pytest.approx(0.14666049094, rel=1e-9)
    assert np.allclose(rec.residual_history, z["residuals"], rtol=1e-6, atol=1e-14)


@pytest.mark.parametrize("kn", [10.0, 1.0, 0.1])
def test_c2_fp64_gmres30_matches_oracle(cuda, kn):
    z, meta = c2_fixture()
    key = f"gmres30_kn{kn:g}"
    rec = Solver(square_case(*C2, tau_r=kn, method="krylov", krylov_restart=30, tol=1e-8, tmax=20000)).run()
    assert rec.converged
    assert abs(rec.iterations - meta[key]["iterations"]) <= 1
    assert rel_l2(rec.temp, z[f"{key}__temp"]) <= 1e-10
    assert rel_l2(rec.qx, z[f"{key}__qx"]) <= 1e-10


def test_c2_cis_matches_oracle(cuda):
    z, meta = c2_fixture()
    rec = Solver(square_case(*C2, tau_r=10.0, tol=1e-8, tmax=20000)).run()
    assert rec.converged
    assert abs(rec.iterations - meta["cis_kn10"]["iterations"]) <= 1
    assert rel_l2(rec.temp, z["cis_kn10__temp"]) <= 1e-10
    assert rel_l2(rec.qx, z["cis_kn10__qx"]) <= 1e-10


def test_c2_gsis_matches_oracle(cuda):
    z, meta = c2_fixture()
    rec = Solver(square_case(*C2, tau_r=0.01, accflag=1, tol=1e-8, tmax=20000)).run()
    assert rec.converged
    assert abs(rec.iterations - meta["gsis_kn0.01"]["iterations"]) <= 1
    assert rel_l2(rec.temp, z["gsis_kn0.01__temp"]) <= 1e-10
    assert rel_l2(rec.qx, z["gsis_kn0.01__qx"]) <= 1e-10


@pytest.mark.parametrize("kn", [10.0, 1.0, 0.1])
def test_c2_mixed_reaches_the_oracle_fixed_point(cuda, kn):
    z, _ = c2_fixture()
    key = f"tight_kn{kn:g}"
    rec = Solver(square_case(*C2, tau_r=kn, method="krylov", krylov_restart=30, tol=1e-8, tmax=20000,
                             precision="mixed")).run()
    assert rec.converged
    assert rel_l2(rec.temp, z[f"{key}__temp"]) <= 1e-8
    # the heat flux as a vector field (q_y alone is ~1e-7 of q_x here: the
    # square is symmetric about y = 1/2)
    assert rel_l2(np.concatenate([rec.qx, rec.qy]), np.concatenate([z[f"{key}__qx"], z[f"{key}__qy"]])) <= 1e-8


def test_c2_mixed_gsis_reaches_the_gsis_fixed_point(cuda):
    """Kn_R = 0.01 (GSIS): the mixed solve against the FP64 GSIS drop-in
    iterated to 1e-13 (the drop-in itself matches the oracle above): the GSIS
    fixed point within 1e-8 relative L2."""
    ref = Solver(square_case(*C2, tau_r=0.01, accflag=1, tol=1e-13, tmax=20000)).run()
    assert ref.converged
    rec = Solver(square_case(*C2, tau_r=0.01, accflag=1, tol=1e-8, tmax=20000, precision="mixed",
                             krylov_restart=30)).run()
    assert rec.converged
    assert rel_l2(rec.temp, ref.temp) <= 1e-8
    assert rel_l2(np.concatenate([rec.qx, rec.qy]), np.concatenate([ref.qx, ref.qy])) <= 1e-8
