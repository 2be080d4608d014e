"""Many uneven cases in one batched sweep launch per DG order, and the
lockstep batched mixed-precision solver built on it: every case's result is
the one it gives solved alone."""
import ctypes

import numpy as np
import pytest
import torch

from pbte_gb300 import Solver, _lib, square_case
from pbte_gb300.batch import LockstepBatch, tune_batch_shape
from pbte_gb300.config import batched_instances
from pbte_gb300.krylov import FixedPointOperator
from pbte_gb300.mixed import run_mixed

pytestmark = pytest.mark.gpu


def uneven(method="krylov"):
    """Five small cases of different grids, orders, ordinate counts, Kn and walls."""
    spec = [(8, 1, 4, 8, 1.0, 0.5), (12, 2, 4, 16, 0.3, 1.0), (6, 3, 2, 8, 2.0, 0.2), (16, 1, 8, 16, 0.1, 0.7),
            (10, 2, 2, 8, 5.0, 0.4)]
    out = []
    for n, deg, npole, nazim, kn, dt in spec:
        kw = dict(tau_r=kn, tau_n=0.1 * kn, tol=1e-8, tmax=20000, t_west=dt, t_east=-dt, precision="mixed",
                  krylov_restart=12)
        if method == "gsis":
            out.append(square_case(n, deg, npole, nazim, accflag=1, **kw))
        else:
            out.append(square_case(n, deg, npole, nazim, method="krylov", **kw))
    return out


def test_batched_sweep_gives_each_cases_single_sweep(cuda):
    """One launch per order over all cases' velocities (several block shapes)
    against each case's own folded FP32 sweep: the same bits."""
    L = _lib.lib()
    solvers = [Solver(c) for c in uneven()]
    ops = [FixedPointOperator(s, "fp32", homogeneous=False, integrals=False) for s in solvers]
    g = torch.Generator(device="cpu").manual_seed(5)
    ref = []
    for op in ops:
        op.uin.copy_(torch.randn(op.n, generator=g, dtype=torch.float64))
        ts, qxs, qys, fw, _ = op._views(op.uin)
        _lib.check(L.pbte_sweep_fold_f32(op.s.ctx.handle, ts.data_ptr(), qxs.data_ptr(), qys.data_ptr(),
                                         op._ptr(fw), 1.0, op.vdf.data_ptr(), None), "sweep_fold_f32")
        torch.cuda.synchronize()
        ref.append(op.vdf.clone())
    items = (_lib.BatchItem * len(ops))(*[op.batch_item(None) for op in ops])
    for shape in ((4, 64), (8, 64), (2, 128), (1, 64)):
        for op in ops:
            op.vdf.zero_()
        h = ctypes.c_void_p()
        _lib.check(L.pbte_sweep_batch_create(len(ops), items, shape[0], shape[1], ctypes.byref(h)), "create")
        _lib.check(L.pbte_sweep_batch_run(h, 1, None), "run")
        torch.cuda.synchronize()
        L.pbte_sweep_batch_destroy(h)
        for op, r in zip(ops, ref):
            assert torch.equal(op.vdf, r), shape


@pytest.mark.parametrize("method", ["krylov", "gsis"])
@pytest.mark.parametrize("graphs", [True, False])
def test_lockstep_batch_gives_the_solo_results(cuda, method, graphs):
    cases = uneven(method)
    solo = []
    for c in cases:
        s = Solver(c)
        solo.append(run_mixed(s))
        s.release()
    batch = LockstepBatch([Solver(c) for c in cases], shape=(4, 64), use_graphs=graphs)
    for _ in range(2):                     # twice: the second run replays the captured chunks
        recs = batch.run()
        for a, b in zip(recs, solo):
            assert a.converged and b.converged
            assert a.diagnostics["fp32_sweeps"] == b.diagnostics["fp32_sweeps"]
            assert a.diagnostics["outer_steps"] == b.diagnostics["outer_steps"]
            assert np.array_equal(a.temp_dofs, b.temp_dofs) and np.array_equal(a.qx_dofs, b.qx_dofs)


def test_batch_autotuner_and_instance_draw(cuda):
    cases = batched_instances(seed=0, count=64)
    assert len(cases) == 64 and {c.dg.deg for c in cases} == {1, 2, 3}
    small = [c for c in batched_instances(seed=0, count=64, method="krylov") if c.mesh.file.endswith(":16")][:4]
    res = tune_batch_shape([Solver(c) for c in small])
    assert tuple(res["choice"]) in {(4, 64), (8, 64), (2, 128), (4, 128)}
    assert all(v > 0 for v in res["ms"].values())
