"""The CPU oracle (oracle/) pinned against the reference: bit-for-bit kernels
when fed the reference's own setup arrays, and exact iteration counts /
fields for complete CIS, GSIS and GMRES(30) solves (golden fixtures made by
tests/golden/make_golden.py from pybte), plus the certified task solutions."""
import numpy as np
import pytest

from cases import case_from_meta, golden, meta, periodic_case, small_case, task_case
from oracle.oracle import Oracle
from pbte_gb300.discretisation import Discretisation
from pbte_gb300.mesh import structured_square


def _oracle_on_reference_arrays(deg):
    z = golden(f"setup_sweep_deg{deg}")
    disc = Discretisation.build(small_case(deg, 4, 8, 0.5, 0.05))
    it = disc.integrals
    for k in ("int_tri", "int_tri_tri", "int_tri_tri_x", "int_tri_tri_y", "int_tri_fc", "int_tri_tri_fc",
              "int_tri_fc_fc"):
        setattr(it, k, np.ascontiguousarray(z[k]))
    o = Oracle(disc, nthreads=2)
    rng = np.random.default_rng(100 + deg)
    o.ts[:] = rng.standard_normal(o.ts.shape)
    o.qxs[:] = 0.3 * rng.standard_normal(o.ts.shape)
    o.qys[:] = 0.3 * rng.standard_normal(o.ts.shape)
    o.vdf[:] = rng.standard_normal(o.vdf.shape)
    return o, z


@pytest.mark.parametrize("deg", [1, 2, 3])
def test_kernels_bitwise_against_reference(deg):
    o, z = _oracle_on_reference_arrays(deg)
    assert np.array_equal(o.order, z["order"])
    assert np.array_equal(o.vdf, z["vdf_in"])
    o.wall_flux()
    assert np.array_equal(o.flux_wall, z["flux_wall"])
    o.sweep()
    # the reference's numpy path factors with LAPACK (scipy's OpenBLAS dgetrf /
    # dgetrs); the oracle restates pybte/_kernels.py's DGETF2 look-alike, which
    # agrees with it to rounding (observed <= 4.3e-16 absolute on O(1) values)
    assert np.abs(o.vdf - z["vdf_out"]).max() <= 1e-14 * np.abs(z["vdf_out"]).max()
    assert o.true_residual() == pytest.approx(float(z["true_residual"]), rel=0.3, abs=1e-15)
    # moments of the reference's own post-sweep distribution: bit for bit
    o.vdf[:] = z["vdf_out"]
    o.moments()
    for k in ("ts", "qxs", "qys", "temp", "qx", "qy"):
        assert np.array_equal(getattr(o, k), z[f"{k}_out"]), k


@pytest.mark.parametrize("name", ["cis_deg1_adiabatic", "cis_deg2_isothermal", "gsis_deg2_adiabatic",
                                  "gsis_deg1_isothermal", "krylov_deg2_adiabatic"])
def test_complete_solves_match_reference(name):
    z = golden(name)
    m = meta()[name]
    o = Oracle(Discretisation.build(case_from_meta(name)), nthreads=2)
    if m.get("method") == "krylov":
        r = o.run_krylov(max_basis=30)
    else:
        r = o.run_source(gsis=bool(m.get("accflag")))
    assert r["iterations"] == int(z["iterations"])
    assert r["converged"]
    assert np.abs(o.temp - z["temp"]).max() <= 1e-12 * np.abs(z["temp"]).max()
    assert np.abs(o.ts - z["ts"]).max() <= 1e-11 * np.abs(z["ts"]).max()
    if m.get("method") != "krylov":   # GMRES iterates amplify rounding; compare only the end
        assert np.allclose(r["masses"], z["masses"], rtol=0, atol=1e-12)
    assert abs(o.mass - float(z["masses"][-1])) < 1e-12


def _periodic_oracle(deg):
    """The oracle on the periodic channel with the fixture's seeded state
    (same draws, same order as make_golden.py)."""
    z = golden("periodic")
    o = Oracle(Discretisation.build(periodic_case(deg, 4, 8, 0.5, 0.05)), nthreads=2)
    rng = np.random.default_rng(200 + deg)
    o.ts[:] = rng.standard_normal(o.ts.shape)
    o.qxs[:] = 0.3 * rng.standard_normal(o.ts.shape)
    o.qys[:] = 0.3 * rng.standard_normal(o.ts.shape)
    o.vdf[:] = rng.standard_normal(o.vdf.shape)
    pbuf = rng.standard_normal(o.pbuf.shape)
    return o, z, pbuf


@pytest.mark.parametrize("deg", [1, 2])
def test_periodic_sweeps_against_reference(deg):
    """Both periodic forms of the reference sweep: the partner read from the
    current distribution (fresh or lagged by its place in TRI_ORDER), and
    from pbuf."""
    o, z, pbuf = _periodic_oracle(deg)
    assert np.array_equal(o.vdf, z[f"deg{deg}_vdf_in"]) and np.array_equal(pbuf, z[f"deg{deg}_pbuf"])
    assert np.array_equal(o.arr["periodic_tri"], z[f"deg{deg}_periodic_tri"])
    vdf0 = o.vdf.copy()
    o.sweep()
    ref = z[f"deg{deg}_vdf_cis"]
    assert np.abs(o.vdf - ref).max() <= 1e-14 * np.abs(ref).max()
    assert o.true_residual() == pytest.approx(float(z[f"deg{deg}_true_residual"]), rel=0.3, abs=1e-15)
    o.vdf[:] = vdf0
    o.pbuf[:] = pbuf
    o.use_pbuf = True
    o.sweep()
    ref = z[f"deg{deg}_vdf_pbuf"]
    assert np.abs(o.vdf - ref).max() <= 1e-14 * np.abs(ref).max()


@pytest.mark.parametrize("name", ["cis_deg1", "gsis_deg2", "krylov_deg2"])
def test_periodic_solves_match_reference(name):
    z = golden("periodic")
    m = meta()[f"periodic_{name}"]
    kw = {k: m[k] for k in ("deg", "npole", "nazim", "tau_r", "tau_n")}
    o = Oracle(Discretisation.build(periodic_case(**kw, accflag=m.get("accflag", 0),
                                                  method=m.get("method", "source"))), nthreads=2)
    if m.get("method") == "krylov":
        r = o.run_krylov(max_basis=30)
        assert abs(r["iterations"] - m["iterations"]) <= 1
    else:
        r = o.run_source(gsis=bool(m.get("accflag")))
        assert r["iterations"] == m["iterations"]
    assert r["converged"]
    tol = 1e-9 if m.get("method") == "krylov" else 1e-12
    assert np.abs(o.temp - z[f"{name}_temp"]).max() <= tol * np.abs(z[f"{name}_temp"]).max()
    assert abs(o.mass - m["mass"]) < 1e-10


def test_shipped_channel_mesh_is_the_structured_generator():
    """pybte's meshes/C1_Nx11_Ny11.msh (the F3 family's periodic channel) is
    the 10 x 10 channel, uniform in x and smootherstep in y."""
    z = golden("periodic")
    raw = structured_square(10, "channel", "smootherstep", "uniform")
    assert np.array_equal(raw.nodes, z["shipped_nodes"])
    assert np.array_equal(raw.tri_nodes, z["shipped_tri_nodes"])
    assert np.array_equal(raw.line_nodes, z["shipped_line_nodes"])
    assert np.array_equal(raw.line_phyid, z["shipped_line_phyid"])


def task_solution(key: str) -> np.ndarray:
    """Certified temperatures of a task cell (F3 lives with the periodic
    fixtures)."""
    if key.startswith("F3"):
        return golden("periodic")[f"task_{key}__temp"]
    return golden("task_solutions")[f"{key}__temp"]


@pytest.mark.parametrize("key", ["F1_1_1", "F1_1e-1", "F2_1_1", "F2_1e-1", "F3_1_1"])
def test_task_certified_solutions(key):
    """The reference task's solutions (GMRES to 1e-10): same sweep count,
    fields within the task's own field-gap bar (1e-5; observed ~1e-12)."""
    fam, tau = key.split("_", 1)
    temp = task_solution(key)
    o = Oracle(Discretisation.build(task_case(fam, tau)), nthreads=4)
    r = o.run_krylov()
    want = meta()[f"task_{key}"]
    assert r["converged"]
    assert abs(r["iterations"] - want["iterations"]) <= 1
    gap = np.abs(o.temp - temp).max() / np.abs(temp).max()
    assert gap < 1e-9
    assert abs(o.mass - want["mass"]) < 1e-10
