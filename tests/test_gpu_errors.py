"""Failure paths on the GPU, none of which faults the device: singular
element operators (pybte raises LinAlgError, ``sweep.py:122-128``), a cyclic
direction (SweepCycleError, ``ordering.py:169``), a NaN in the state (the
solve ends unconverged at tmax instead of hanging), and the reference task
verifier's own calls (``tasks/t01-square/verifier/run_agent_case.py:69-92``).
A failed context creation frees every device byte it took."""
import ctypes
import types

import numpy as np
import pytest
import torch

from cases import small_case
from pbte_gb300 import Solver, SweepCycleError, _lib
from pbte_gb300.discretisation import Discretisation
from pbte_gb300.sweep import SweepContext
from test_errors import cyclic_disc

pytestmark = pytest.mark.gpu


def _live() -> int:
    v = ctypes.c_int64(-1)
    _lib.check(_lib.lib().pbte_device_bytes_live(ctypes.byref(v)), "device_bytes_live")
    return int(v.value)


def _singular_disc(**kw):
    """Element 0 with no area and no edges: its operator is the zero matrix."""
    disc = Discretisation.build(small_case(1, 4, 8, 0.5, 0.05, **kw))
    it = disc.integrals
    for a in (it.area2, it.dxi, it.deta, it.edge_scale):
        a[0] = 0.0
    return disc


def test_singular_operator_raises_at_setup_and_frees_its_memory(cuda):
    before = _live()
    with pytest.raises(np.linalg.LinAlgError):
        SweepContext(_singular_disc(), precompute=True)
    assert _live() == before


def test_singular_operator_in_onthefly_sweeps_raises_after_the_run(cuda):
    disc = _singular_disc(tmax=6, sweep_mode="onthefly")
    s = Solver(disc.case, discretisation=disc)
    assert s.ctx.mode == "onthefly"
    with pytest.raises(np.linalg.LinAlgError):
        s.run()
    assert s.ctx.singular_count() == 0           # the run's count was read and reset


def test_cyclic_direction_raises_and_frees_its_memory(cuda):
    disc, _ = cyclic_disc()
    before = _live()
    with pytest.raises(SweepCycleError):
        SweepContext(disc)
    assert _live() == before


@pytest.mark.parametrize("method", ["source", "krylov"])
def test_nan_state_ends_unconverged_at_tmax(cuda, method):
    s = Solver(small_case(1, 4, 8, 0.5, 0.05, method=method, tmax=40, krylov_restart=8))
    s.mom.ts[0, 0] = float("nan")
    if method == "krylov":
        s.vdf[0, 0, 0] = float("nan")
        s.restart_info = {"enabled": True}       # start GMRES from this state
    rec = s.run()
    assert not rec.converged
    assert rec.iterations <= 40


def test_verifier_calls(cuda):
    """The verifier's sequence on a solver: run, save np.asarray(solver.vdf),
    then time solver.ctx.sweep(solver.mom, solver.vdf); and the same sweep
    with host numpy moments and distribution gives the device result."""
    s = Solver(small_case(2, 4, 8, 0.5, 0.05))
    rec = s.run()
    assert rec.converged
    host = np.asarray(s.vdf)
    assert isinstance(host, np.ndarray) and host.shape == tuple(s.vdf.shape)
    assert np.array_equal(host, s.vdf.detach().cpu().numpy())
    for _ in range(3):
        s.ctx.sweep(s.mom, s.vdf)
    torch.cuda.synchronize()
    dev = s.vdf.detach().cpu().numpy()
    mom = types.SimpleNamespace(**{k: getattr(s.mom, k).cpu().numpy() for k in ("ts", "qxs", "qys")})
    v = host.copy()
    for _ in range(3):
        s.ctx.sweep(mom, v)
    assert np.array_equal(v, dev)
