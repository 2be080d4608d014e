"""GPU parity: the CUDA path (through the C ABI) against the CPU oracle on the
same inputs, and against the reference's golden solves.

Tolerances: FP64 kernels 1e-11 relative.  The GPU forms the element operators
from the compact reference matrices (the neighbour coupling as an edge gather,
which differs from the reference's 15-point quadrature tensor by ~3e-13) and
factors with reciprocal pivots, so it differs from the oracle by rounding
only: observed 1.1e-12 (P1) to 2.3e-12 (P3); complete FP64 solves 1e-10 on the
fields with the iteration count exact or within 1; the mixed path 1e-8
against the FP64 fixed point.
"""
import numpy as np
import pytest
import torch

from cases import case_from_meta, golden, meta, small_case, task_case
from oracle.oracle import Oracle
from pbte_gb300 import Solver
from pbte_gb300.config import square_case

pytestmark = pytest.mark.gpu


def _rel(a, b):
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))


def _seed_state(s, o, seed):
    rng = np.random.default_rng(seed)
    for k in ("ts", "qxs", "qys"):
        v = rng.standard_normal(getattr(o, k).shape) * (1.0 if k == "ts" else 0.3)
        getattr(o, k)[:] = v
        getattr(s.mom, k).copy_(torch.from_numpy(v))
    o.vdf[:] = rng.standard_normal(o.vdf.shape)
    s.vdf.copy_(torch.from_numpy(o.vdf))


@pytest.mark.parametrize("deg", [1, 2, 3])
@pytest.mark.parametrize("mode", ["precomputed", "onthefly"])
@pytest.mark.parametrize("south", ["nonthermalising", "thermalising"])
def test_sweep_moments_flux_match_oracle(cuda, deg, mode, south):
    case = small_case(deg, 4, 8, 0.5, 0.05, south=south, sweep_mode=mode)
    s = Solver(case)
    assert s.ctx.mode == mode
    o = Oracle(s.disc, nthreads=4)
    _seed_state(s, o, 7 + deg)
    o.wall_flux()
    s.ctx.wall_flux(s.vdf)
    torch.cuda.synchronize()
    if south == "nonthermalising":
        assert _rel(s.ctx.flux_wall.cpu().numpy(), o.flux_wall) < 1e-11
    o.sweep()
    s.ctx.sweep(s.mom, s.vdf)
    torch.cuda.synchronize()
    assert _rel(s.vdf.cpu().numpy(), o.vdf) < 1e-11
    o.moments()
    s.ctx.moments(s.vdf, s.mom)
    h = s.mom.host()
    for k in ("ts", "qxs", "qys", "temp", "qx", "qy"):
        assert _rel(h[k], getattr(o, k)) < 1e-11, k
    tr_o = o.true_residual()
    tr_g = s.ctx.true_residual(s.mom, s.vdf)
    assert abs(tr_g - tr_o) < 1e-9 * max(tr_o, 1e-12) + 1e-14


@pytest.mark.parametrize("deg", [1, 2, 3])
def test_ring_sweep_chunks_levels_wider_than_its_registers(cuda, deg):
    """Levels wider than a thread group holds in registers run in chunks (only
    the first waits for the level before, only the last hands the level on):
    a 136 x 136 square (levels 136 wide; P3: 72 x 72, levels 72 wide, whose
    groups hold one element per thread) swept with block shapes whose groups
    hold 64 or 128 elements, FP64 and FP32, against the oracle."""
    n = 72 if deg == 3 else 136
    s = Solver(small_case(deg, 2, 8, 0.3, 0.03, mesh=f"cavity:{n}", sweep_mode="onthefly"))
    assert s.ctx.schedule()["ring_W"] > (64 if deg == 3 else 128)
    o = Oracle(s.disc, nthreads=4)
    _seed_state(s, o, 23)
    o.wall_flux()
    s.ctx.wall_flux(s.vdf)
    o.sweep()
    s.ctx.set_variant(2)
    shapes = [(1, 64), (2, 64), (4, 64), (8, 64), (1, 128), (2, 128), (4, 128)]
    for g, w in shapes:
        s.ctx.set_groups(g, w)
        v = s.vdf.clone()
        s.ctx.sweep(s.mom, v)
        u = torch.zeros(s.vdf.shape, dtype=torch.float32, device=s.device)
        s.ctx.sweep_f32((s.mom.ts, s.mom.qxs, s.mom.qys), u, s.ctx.flux_wall)
        torch.cuda.synchronize()
        assert _rel(v.cpu().numpy(), o.vdf) < 1e-11, (g, w)
        assert _rel(u.double().cpu().numpy(), o.vdf) < 2e-5, (g, w)
    s.ctx.set_groups(0, 0)
    s.ctx.set_variant(0)


@pytest.mark.parametrize("deg", [1, 2, 3])
@pytest.mark.parametrize("mode", ["precomputed", "onthefly"])
def test_ring_and_level_serial_sweeps_agree(cuda, deg, mode):
    """The ring-pipelined kernel (one block per in-plane velocity, twins
    stored from one solve) against the level-serial kernel and the oracle,
    on a 40 x 40 square (FP64 ring in shared memory) and, for FP32, on a
    72 x 72 square (levels 72 wide: two cells per thread)."""
    mesh = "cavity:40" if deg < 3 else "cavity:24"
    case = small_case(deg, 4, 8, 0.3, 0.03, mesh=mesh, sweep_mode=mode)
    s = Solver(case)
    o = Oracle(s.disc, nthreads=4)
    _seed_state(s, o, 21)
    o.wall_flux()
    s.ctx.wall_flux(s.vdf)
    o.sweep()
    out = {}
    for variant in (1, 2):
        s.ctx.set_variant(variant)
        v = s.vdf.clone()
        s.ctx.sweep(s.mom, v)
        torch.cuda.synchronize()
        out[variant] = v.cpu().numpy()
        assert _rel(out[variant], o.vdf) < 1e-11, variant
    if mode == "onthefly":
        if deg < 3:
            s = Solver(small_case(deg, 4, 8, 0.3, 0.03, mesh="cavity:72", sweep_mode=mode))
            assert s.ctx.schedule()["ring_W"] > 64
            o = Oracle(s.disc, nthreads=4)
            _seed_state(s, o, 22)
            o.wall_flux()
            s.ctx.wall_flux(s.vdf)
            o.sweep()
        v32 = {}
        for variant in (1, 2):
            s.ctx.set_variant(variant)
            w = torch.zeros(s.vdf.shape, dtype=torch.float32, device=s.device)
            s.ctx.sweep_f32((s.mom.ts, s.mom.qxs, s.mom.qys), w, s.ctx.flux_wall)
            torch.cuda.synchronize()
            v32[variant] = w.double().cpu().numpy()
            assert _rel(v32[variant], o.vdf) < 2e-5, variant
    s.ctx.set_variant(0)


@pytest.mark.parametrize("deg", [1, 2, 3])
def test_transport_residual_of_random_state(cuda, deg):
    s = Solver(small_case(deg, 4, 8, 0.2, 0.02))
    o = Oracle(s.disc, nthreads=4)
    _seed_state(s, o, 3)
    o.wall_flux()
    s.ctx.wall_flux(s.vdf)
    assert s.ctx.true_residual(s.mom, s.vdf) == pytest.approx(o.true_residual(), rel=1e-11)


def test_fp32_sweep_close_to_fp64(cuda):
    s = Solver(small_case(2, 4, 8, 0.5, 0.05))
    o = Oracle(s.disc, nthreads=4)
    _seed_state(s, o, 11)
    o.wall_flux()
    o.sweep()
    s.ctx.wall_flux(s.vdf)
    v32 = torch.zeros(s.vdf.shape, dtype=torch.float32, device=s.device)
    # FP32 sweeps overwrite every element, so the upwind inflow comes from this sweep
    s.ctx.sweep_f32((s.mom.ts, s.mom.qxs, s.mom.qys), v32, s.ctx.flux_wall)
    torch.cuda.synchronize()
    assert _rel(v32.double().cpu().numpy(), o.vdf) < 2e-5


@pytest.mark.parametrize("deg", [1, 2, 3])
@pytest.mark.parametrize("mesh", ["cavity:5:smootherstep", "cavity:40"])
def test_stored_fp32_factors_match_register_factorisation(cuda, deg, mesh):
    """FP32 sweeps with the factors stored by pbte_factorise_f32 against the
    same sweeps factoring in registers: the factoriser uses the sweep's own
    FP32 arithmetic, so the two agree to FP32 rounding (bit for bit where the
    compiler contracts both alike)."""
    s = Solver(small_case(deg, 4, 8, 0.5, 0.05, mesh=mesh))
    assert not s.ctx.fp32_factors
    o = Oracle(s.disc, nthreads=4)
    _seed_state(s, o, 13)
    s.ctx.wall_flux(s.vdf)
    out = []
    for stored in (False, True):
        if stored:
            s.ctx.factorise_f32()
        v32 = torch.zeros(s.vdf.shape, dtype=torch.float32, device=s.device)
        s.ctx.sweep_f32((s.mom.ts, s.mom.qxs, s.mom.qys), v32, s.ctx.flux_wall)
        torch.cuda.synchronize()
        out.append(v32.double().cpu().numpy())
    assert _rel(out[1], out[0]) < 1e-6
    o.wall_flux()
    o.sweep()
    assert _rel(out[1], o.vdf) < 2e-5


@pytest.mark.parametrize("deg", [1, 2, 3])
def test_fused_fp32_product_matches_separate_calls(cuda, deg):
    """pbte_fixed_point_f32 (sources, sweep, moments and emission in one call,
    z-mirror twins folded) against pbte_sweep_f32 + pbte_moments_f32 +
    pbte_wall_flux_f32 on every ordinate: the same numbers up to the FP32
    rounding of w_a f + w_b f against (w_a + w_b) f (tolerance 1e-6)."""
    from pbte_gb300 import _lib
    s = Solver(small_case(deg, 4, 8, 0.5, 0.05))
    o = Oracle(s.disc, nthreads=4)
    _seed_state(s, o, 21)
    s.ctx.wall_flux(s.vdf)
    L, st = _lib.lib(), torch.cuda.current_stream().cuda_stream
    h, m = s.ctx.handle, s.mom
    f64 = dict(dtype=torch.float64, device="cuda")
    v32 = torch.zeros(s.vdf.shape, dtype=torch.float32, device="cuda")
    ref = [torch.zeros_like(m.ts) for _ in range(3)] + [torch.zeros_like(s.ctx.flux_wall)]
    out = [torch.zeros_like(m.ts) for _ in range(3)] + [torch.zeros_like(s.ctx.flux_wall)]
    ints = [torch.zeros(s.n_tris, **f64) for _ in range(6)]
    _lib.check(L.pbte_sweep_f32(h, m.ts.data_ptr(), m.qxs.data_ptr(), m.qys.data_ptr(), v32.data_ptr(),
                                s.ctx.flux_wall.data_ptr(), 1.0, st), "sweep_f32")
    _lib.check(L.pbte_moments_f32(h, v32.data_ptr(), *(r.data_ptr() for r in ref[:3]),
                                  *(i.data_ptr() for i in ints[:3]), st), "moments_f32")
    _lib.check(L.pbte_wall_flux_f32(h, v32.data_ptr(), ref[3].data_ptr(), st), "wall_flux_f32")
    v32.zero_()
    _lib.check(L.pbte_fixed_point_f32(h, m.ts.data_ptr(), m.qxs.data_ptr(), m.qys.data_ptr(),
                                      s.ctx.flux_wall.data_ptr(), 1.0, v32.data_ptr(),
                                      *(x.data_ptr() for x in out), *(i.data_ptr() for i in ints[3:]), st),
               "fixed_point_f32")
    torch.cuda.synchronize()
    for a, b in zip(out + ints[3:], ref + ints[:3]):
        assert _rel(a.cpu().numpy(), b.cpu().numpy()) < 1e-6


@pytest.mark.parametrize("name", ["cis_deg1_adiabatic", "cis_deg2_isothermal"])
def test_cis_solve_matches_reference(cuda, name):
    z = golden(name)
    s = Solver(case_from_meta(name))
    rec = s.run()
    assert rec.converged
    assert rec.iterations == int(z["iterations"])
    assert _rel(rec.temp, z["temp"]) < 1e-10
    assert _rel(rec.temp_dofs, z["ts"]) < 1e-10
    assert _rel(rec.qx_dofs, z["qxs"]) < 1e-9
    assert np.allclose(rec.residual_history, z["residuals"], rtol=1e-6, atol=1e-14)


def test_cis_graph_stops_at_tmax(cuda):
    s = Solver(small_case(1, 4, 8, 1.0, 0.1, tmax=45), graph_block=32)
    rec = s.run()
    assert rec.iterations == 45 and not rec.converged


@pytest.mark.parametrize("name", ["gsis_deg2_adiabatic", "gsis_deg1_isothermal"])
def test_gsis_solve_matches_reference(cuda, name):
    z = golden(name)
    s = Solver(case_from_meta(name))
    rec = s.run()
    assert rec.converged
    assert abs(rec.iterations - int(z["iterations"])) <= 1
    assert _rel(rec.temp, z["temp"]) < 1e-10
    assert _rel(rec.temp_dofs, z["ts"]) < 1e-10


def test_krylov_gmres30_matches_reference(cuda):
    name = "krylov_deg2_adiabatic"
    z = golden(name)
    s = Solver(case_from_meta(name, krylov_restart=30))
    rec = s.run()
    assert rec.converged
    assert abs(rec.iterations - int(z["iterations"])) <= max(1, int(0.02 * int(z["iterations"])))
    assert _rel(rec.temp, z["temp"]) < 1e-8
    assert rec.diagnostics["transport_residual"] < 1e-8


@pytest.mark.parametrize("key", ["F1_1_1", "F2_1e-1"])
def test_task_certified_solution(cuda, key):
    fam, tau = key.split("_", 1)
    sol = golden("task_solutions")
    rec = Solver(task_case(fam, tau)).run()
    assert rec.converged
    assert abs(rec.iterations - meta()[f"task_{key}"]["iterations"]) <= 1
    assert _rel(rec.temp, sol[f"{key}__temp"]) < 1e-9


@pytest.mark.parametrize("method", ["source", "krylov"])
def test_mixed_precision_reaches_fp64_fixed_point(cuda, method):
    base = dict(deg=2, npole=4, nazim=8, tau_r=0.2, tau_n=0.02)
    o = Oracle(Solver(small_case(**base)).disc, nthreads=4)
    r = o.run_krylov(tol=1e-13, tmax=5000)
    assert r["converged"]
    s = Solver(small_case(**base, method=method, precision="mixed"))
    rec = s.run()
    assert rec.converged
    assert _rel(rec.temp_dofs, o.ts) < 1e-8
    assert _rel(rec.qx_dofs, o.qxs) < 1e-8
    assert rec.diagnostics["fp32_sweeps"] > rec.diagnostics["fp64_sweeps"]


@pytest.mark.parametrize("name", ["gsis_deg2_adiabatic", "gsis_deg1_isothermal"])
def test_fp32_gsis_product_is_the_linear_part_of_the_gsis_step(cuda, name):
    """The FP64 GSIS step as a map on the sweep inputs, G(u) = T u + g, is the
    same captured or launched directly; and the FP32 GSIS product of the mixed
    solve (homogeneous: walls at zero temperature) is its linear part T to
    FP32 accuracy: G(u) - G(v) = T32 (u - v) within 1e-5."""
    from pbte_gb300.gsis import GsisFixedPoint
    out = {}
    for graphs in (True, False):
        s = Solver(case_from_meta(name, precision="mixed"))
        s.use_graphs = graphs
        op64, op32 = GsisFixedPoint(s, "fp64"), GsisFixedPoint(s, "fp32", homogeneous=True)
        g = torch.Generator(device="cpu").manual_seed(3)
        u = torch.randn(op64.n, generator=g, dtype=torch.float64).to(cuda)
        v = torch.randn(op64.n, generator=g, dtype=torch.float64).to(cuda)
        gu, gv = op64.apply(u), op64.apply(v)
        t = op32.apply(u - v)
        assert float((gu - gv - t).norm() / t.norm()) < 1e-5
        out[graphs] = (gu, gv, t)
    for a, b in zip(out[True], out[False]):
        assert float((a - b).norm() / b.norm()) < 1e-12


@pytest.mark.parametrize("name", ["gsis_deg2_adiabatic", "gsis_deg1_isothermal"])
@pytest.mark.parametrize("graphs", [True, False])
def test_mixed_gsis_reaches_the_gsis_fixed_point(cuda, name, graphs):
    """Mixed-precision GSIS (FP64 GSIS defects, inner GMRES on FP32 GSIS
    products with the FP64 trace solve) against the oracle's GSIS iterated to
    1e-13: the GSIS fixed point (not CIS's) within 1e-8."""
    o = Oracle(Solver(case_from_meta(name)).disc, nthreads=4)
    r = o.run_source(tol=1e-13, tmax=20000, gsis=True)
    assert r["converged"]
    s = Solver(case_from_meta(name, precision="mixed"))
    s.use_graphs = graphs
    rec = s.run()
    assert rec.converged and rec.scheme == "GSIS"
    assert rec.diagnostics["fp32_sweeps"] > 0
    assert _rel(rec.temp_dofs, o.ts) < 1e-8
    assert _rel(rec.qx_dofs, o.qxs) < 1e-8


@pytest.mark.parametrize("graphs", [True, False])
@pytest.mark.parametrize("basis", [8, 100])
def test_fp64_device_gmres_matches_oracle(cuda, graphs, basis):
    """The FP64 Krylov solve with whole restart cycles on the device (CGS2,
    rotations, the target and pybte's bounded extension tested per column on
    the device, captured in chunks or launched directly) against the oracle's
    restatement of pybte's host loop (``krylov.py:150-363``): the same sweep
    count within one, the same fields to 1e-10.  A basis of 100 vectors
    takes the CGS2 past 64 rows."""
    base = dict(deg=2, npole=4, nazim=8, tau_r=0.2, tau_n=0.02, method="krylov", krylov_restart=basis)
    s = Solver(small_case(**base))
    s.use_graphs = graphs
    rec = s.run()
    o = Oracle(s.disc, nthreads=4)
    r = o.run_krylov(max_basis=basis)
    assert rec.converged and r["converged"]
    assert abs(rec.iterations - r["iterations"]) <= 1
    assert _rel(rec.temp, o.temp) < 1e-10
    assert _rel(rec.qx, o.qx) < 1e-10
    n = min(rec.iterations, r["iterations"]) - 1
    assert np.allclose(rec.residual_history[:n], r["residuals"][:n], rtol=1e-6, atol=1e-13)


@pytest.mark.parametrize("graphs", [True, False])
def test_native_gmres_columns_issue_the_same_launches(cuda, monkeypatch, graphs):
    """The mixed solve's inner cycles with each chunk issued by one native
    call (pbte_gmres_columns_f32: the rotation in the CGS2 norm pass, the
    next sources with the basis update) against the separate calls issued
    column by column from Python, captured or direct: the same arithmetic,
    bit for bit the same solve."""
    from pbte_gb300.krylov import ArnoldiGraphs
    base = dict(deg=2, npole=4, nazim=8, tau_r=0.2, tau_n=0.02, method="krylov", precision="mixed",
                krylov_restart=12)
    out = {}
    for native in (True, False):
        monkeypatch.setattr(ArnoldiGraphs, "native_columns", native)
        s = Solver(small_case(**base))
        s.use_graphs = graphs
        out[native] = s.run()
        s.release()
    a, b = out[True], out[False]
    assert a.converged and b.converged
    assert a.diagnostics["fp32_sweeps"] == b.diagnostics["fp32_sweeps"] > 0
    assert a.iterations == b.iterations
    assert np.array_equal(a.temp_dofs, b.temp_dofs) and np.array_equal(a.qx_dofs, b.qx_dofs)


@pytest.mark.parametrize("m", [21, 42, 70, 105])
def test_batched_inverse_sizes(cuda, m):
    """The HDG element inverses (7 N_p: P1 21 ... P4 105) against LAPACK."""
    from pbte_gb300 import _lib
    rng = np.random.default_rng(m)
    a = rng.standard_normal((9, m, m)) + m * np.eye(m)
    ad = torch.from_numpy(a).to(cuda)
    inv = torch.empty_like(ad)
    bad = torch.zeros(1, dtype=torch.int32, device=cuda)
    _lib.check(_lib.lib().pbte_batched_inverse(ad.data_ptr(), inv.data_ptr(), 9, m, bad.data_ptr(), None),
               "batched_inverse")
    assert int(bad.item()) == 0
    assert _rel(inv.cpu().numpy(), np.linalg.inv(a)) < 1e-12


def test_square_benchmark_mesh_levels(cuda):
    s = Solver(square_case(64, 2, 8, 32, tau_r=1.0, tmax=3))
    assert s.n_tris == 8192
    assert s.ctx.n_classes <= 16
    rec = s.run()
    assert rec.iterations == 3


@pytest.mark.parametrize("rows", [1, 5, 30, 64, 65, 200])
@pytest.mark.parametrize("f32", [False, True])
def test_cgs2_matches_two_pass_gram_schmidt(cuda, rows, f32):
    """pbte_cgs2 / pbte_cgs2_f32 against pybte's CGS2 step
    (pybte/krylov.py:201-210) in numpy, on the same scratch twice in a row
    (the cross-block ticket must be back at zero after each call).  FP64:
    1e-12.  FP32 basis: the numpy reference runs on the FP32-rounded basis
    and vector in FP64; FP32 products and warp sums leave ~1e-6."""
    from pbte_gb300 import _lib
    rng = np.random.default_rng(rows)
    n = 100_003
    Q, _ = np.linalg.qr(rng.standard_normal((n, rows)))
    Q = np.ascontiguousarray(Q.T)
    w = rng.standard_normal(n)
    dt = torch.float32 if f32 else torch.float64
    if f32:
        Q = Q.astype(np.float32).astype(np.float64)
        w = w.astype(np.float32).astype(np.float64)
    c1 = Q @ w
    w1 = w - Q.T @ c1
    c2 = Q @ w1
    w2 = w1 - Q.T @ c2
    scr = torch.zeros(_lib.cgs2_scratch(rows), dtype=torch.float64, device="cuda")
    fn = _lib.lib().pbte_cgs2_f32 if f32 else _lib.lib().pbte_cgs2
    tol = 2e-5 if f32 else 1e-12
    for _ in range(2):
        Qd = torch.from_numpy(Q).to("cuda", dt)
        wd = torch.from_numpy(w).to("cuda", dt)
        h = torch.zeros(rows + 1, dtype=torch.float64, device="cuda")
        _lib.check(fn(Qd.data_ptr(), n, rows, wd.data_ptr(), n, h.data_ptr(), scr.data_ptr(), scr.numel(),
                      torch.cuda.current_stream().cuda_stream), "pbte_cgs2")
        hh = h.cpu().numpy()
        scale = np.linalg.norm(w)
        assert np.abs(hh[:rows] - (c1 + c2)).max() <= tol * scale
        assert hh[rows] == pytest.approx(np.linalg.norm(w2), rel=tol, abs=tol * scale)
        assert np.abs(wd.double().cpu().numpy() - w2).max() <= tol * scale


@pytest.mark.parametrize("f32", [False, True])
@pytest.mark.parametrize("with_g", [False, True])
def test_arnoldi_column_forms_product_then_cgs2(cuda, f32, with_g):
    """pbte_arnoldi_column(_f32): w = q_j - (uout - g), then CGS2 -- the same
    numbers as the separate subtraction followed by pbte_cgs2(_f32)."""
    from pbte_gb300 import _lib
    rng = np.random.default_rng(7)
    n, rows = 50_001, 12
    dt = torch.float32 if f32 else torch.float64
    Q = torch.from_numpy(np.linalg.qr(rng.standard_normal((n, rows)))[0].T.copy()).to("cuda", dt)
    uout = torch.from_numpy(rng.standard_normal(n + 7)).cuda()
    g = torch.from_numpy(rng.standard_normal(n)).cuda() if with_g else None
    L = _lib.lib()
    s = torch.cuda.current_stream().cuda_stream
    w_ref = (Q[rows - 1].double() - (uout[:n] - g if with_g else uout[:n])).to(dt)
    h_ref = torch.zeros(rows + 1, dtype=torch.float64, device="cuda")
    scr = torch.zeros(_lib.CGS2_SCRATCH, dtype=torch.float64, device="cuda")
    cg = L.pbte_cgs2_f32 if f32 else L.pbte_cgs2
    _lib.check(cg(Q.data_ptr(), n, rows, w_ref.data_ptr(), n, h_ref.data_ptr(), scr.data_ptr(), scr.numel(), s),
               "cgs2")
    w = torch.zeros(n, dtype=dt, device="cuda")
    h = torch.zeros(rows + 1, dtype=torch.float64, device="cuda")
    ac = L.pbte_arnoldi_column_f32 if f32 else L.pbte_arnoldi_column
    _lib.check(ac(Q.data_ptr(), n, rows, uout.data_ptr(), g.data_ptr() if with_g else None, w.data_ptr(), n,
                  h.data_ptr(), scr.data_ptr(), scr.numel(), None, s), "arnoldi_column")
    assert torch.equal(w, w_ref)
    assert torch.equal(h, h_ref)
