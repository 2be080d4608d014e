"""The serving loop (pbte_gb300.serve): admission by slots and HBM budget on
the host (CPU, fake runner), and on the GPU that every request's result in
the mix equals the same case solved alone."""
import threading
import time

import numpy as np
import pytest

from pbte_gb300.config import square_case
from pbte_gb300.serve import Server, draw_cases, estimate_device_bytes


def _small(kn, deg=1, n=6, precision="mixed", dt=0.5):
    # 4 x 8 ordinates: with 2 x 4 GMRES stalls on these walls in FP64 as well
    return square_case(n, deg, 4, 8, tau_r=kn, tau_n=0.1 * kn, method="krylov", precision=precision,
                       krylov_restart=30, tol=1e-8, tmax=4000, t_west=dt, t_east=-dt)


class _FakeRunner:
    """Records how many requests run at once and how much budget they hold."""

    def __init__(self, server_ref, hold=0.05):
        self.server_ref, self.hold = server_ref, hold
        self.lock = threading.Lock()
        self.running = self.max_running = 0
        self.order = []

    def __call__(self, case, disc):
        with self.lock:
            self.running += 1
            self.max_running = max(self.max_running, self.running)
            self.order.append(case.flow.tau_r)
            assert self.server_ref[0]._used <= self.server_ref[0].budget
        time.sleep(self.hold)
        with self.lock:
            self.running -= 1
        return case.flow.tau_r


def test_admission_respects_slots_budget_and_arrival_order():
    ref = [None]
    runner = _FakeRunner(ref)
    # every request "needs" 40 units of a 100-unit budget: at most two at once
    srv = Server(device="cpu", hbm_budget=100, slots=3, runner=runner, estimator=lambda d, c: 40)
    ref[0] = srv
    kns = [10.0, 5.0, 2.0, 1.0, 0.5, 0.2]
    tickets = [srv.submit(_small(k)) for k in kns]
    srv.close()
    assert [t.result(timeout=10) for t in tickets] == kns
    assert runner.max_running == 2            # budget-bound, not slot-bound
    assert runner.order == kns                # first come, first admitted
    st = srv.stats()
    assert st["completed"] == len(kns) and st["failed"] == 0 and st["peak_concurrent"] == 2
    assert all(t.admitted >= t.arrival and t.done >= t.admitted for t in tickets)


def test_oversized_request_fails_alone():
    srv = Server(device="cpu", hbm_budget=100, slots=2, runner=lambda c, d: 1.0,
                 estimator=lambda d, c: 500 if c.flow.tau_r == 1.0 else 10)
    a, b = srv.submit(_small(1.0)), srv.submit(_small(2.0))
    srv.close()
    with pytest.raises(MemoryError):
        a.result(timeout=10)
    assert b.result(timeout=10) == 1.0


def test_memory_estimate_grows_with_the_case():
    from pbte_gb300.discretisation import Discretisation
    small, big = _small(1.0, deg=1, n=6), _small(1.0, deg=2, n=12)
    e1 = estimate_device_bytes(Discretisation.build(small), small)
    e2 = estimate_device_bytes(Discretisation.build(big), big)
    assert 0 < e1 < e2


def test_drawn_instances_are_seeded():
    a, b = draw_cases(5, seed=1), draw_cases(5, seed=1)
    assert [c.flow.tau_r for c in a] == [c.flow.tau_r for c in b]
    assert all(1e-3 <= c.flow.tau_r <= 10 for c in a)


@pytest.mark.gpu
def test_results_in_the_mix_equal_results_alone(cuda):
    from pbte_gb300 import Solver
    cases = [_small(10.0, deg=1), _small(1.0, deg=2, n=8), _small(0.5, deg=1, n=10, precision="fp64"),
             _small(2.0, deg=2, n=6, dt=0.3)]
    alone = []
    for c in cases:
        s = Solver(c)
        alone.append(s.run())
        s.release()
    srv = Server(hbm_budget=8e9, slots=3)
    tickets = [srv.submit(c) for c in cases]
    srv.close()
    for t, ref in zip(tickets, alone):
        rec = t.result(timeout=600)
        assert rec.converged and rec.iterations == ref.iterations
        assert np.array_equal(rec.temp, ref.temp) and np.array_equal(rec.qx, ref.qx)
    st = srv.stats()
    assert st["completed"] == len(cases) and st["peak_concurrent"] >= 2


def test_oversized_request_arriving_mid_mix_fails_alone():
    """A request over the whole budget that arrives while others run is
    refused at once; the running and later requests complete."""
    ref = [None]
    runner = _FakeRunner(ref, hold=0.2)
    srv = Server(device="cpu", hbm_budget=100, slots=3, runner=runner,
                 estimator=lambda d, c: 1000 if c.flow.tau_r == 7.0 else 30)
    ref[0] = srv
    first = [srv.submit(_small(k)) for k in (10.0, 5.0)]
    time.sleep(0.05)                            # both running now
    big = srv.submit(_small(7.0))
    last = srv.submit(_small(2.0))
    srv.close()
    with pytest.raises(MemoryError):
        big.result(timeout=10)
    assert big.done < first[0].done             # refused without waiting for the mix
    assert [t.result(timeout=10) for t in first + [last]] == [10.0, 5.0, 2.0]


@pytest.mark.gpu
def test_continuous_batching_results_equal_results_alone(cuda):
    """Lockstep serving: requests arriving over time join the running batch
    between its steps (their FP32 sweeps share the batch's launches), an
    over-budget request arriving mid-mix is refused alone, and every result
    equals the case's solo mixed-precision solve bit for bit."""
    from pbte_gb300 import Solver
    from pbte_gb300.mixed import run_mixed

    cases = [_small(10.0, deg=1), _small(1.0, deg=2, n=8), _small(0.5, deg=1, n=10),
             square_case(8, 2, 4, 8, tau_r=0.05, tau_n=0.005, accflag=1, precision="mixed", tol=1e-8,
                         tmax=4000, krylov_restart=12), _small(2.0, deg=2, n=6, dt=0.3)]
    alone = []
    for c in cases:
        s = Solver(c)
        alone.append(run_mixed(s))
        s.release()
    big = square_case(12, 1, 2, 4, tau_r=1.0, method="krylov", precision="mixed")
    est = lambda d, c: int(50e9) if c is big else int(estimate_device_bytes(d, c))   # noqa: E731
    srv = Server(hbm_budget=40e9, slots=4, mode="lockstep", estimator=est)
    tickets = []
    for i, c in enumerate(cases):
        tickets.append(srv.submit(c))
        if i == 1:
            refused = srv.submit(big)
        time.sleep(0.2)
    srv.close()
    with pytest.raises(MemoryError):
        refused.result(timeout=600)
    for t, ref in zip(tickets, alone):
        rec = t.result(timeout=600)
        assert rec.converged
        assert rec.diagnostics["fp32_sweeps"] == ref.diagnostics["fp32_sweeps"]
        assert np.array_equal(rec.temp_dofs, ref.temp_dofs) and np.array_equal(rec.qx_dofs, ref.qx_dofs)
    assert srv.stats()["completed"] == len(cases)
