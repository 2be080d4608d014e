"""The allocation-free transport residual (``pbte_transport_residual_noalloc``).

It serves callers that cannot allocate device memory where they call from --
hosts whose device memory is handed out by their own pool, so that a
cudaMalloc behind their back fails or breaks their accounting -- by keeping its
scratch in a static device array instead of the context's buffers.  Checked here through the C ABI
against ``pbte_transport_residual`` on the same state, on two calls in a row
with different states (so stale scratch would show), and for the size and
periodic-face limits.
This file is collected last so that a failure here leaves every other test
already run.
"""
import ctypes

import numpy as np
import pytest
import torch

from cases import periodic_case, small_case
from pbte_gb300 import Solver, _lib

pytestmark = pytest.mark.gpu


def _seed(s, seed):
    g = torch.Generator(device="cpu").manual_seed(seed)
    for k in ("ts", "qxs", "qys"):
        getattr(s.mom, k).copy_(torch.randn(getattr(s.mom, k).shape, generator=g, dtype=torch.float64))
    s.vdf.copy_(torch.randn(s.vdf.shape, generator=g, dtype=torch.float64))
    s.ctx.wall_flux(s.vdf)


def _live_bytes() -> int:
    v = ctypes.c_int64(-1)
    _lib.check(_lib.lib().pbte_device_bytes_live(ctypes.byref(v)), "device_bytes_live")
    return int(v.value)


def _call(fn, s, num, den, *extra):
    m = s.mom
    st = torch.cuda.current_stream().cuda_stream
    args = [s.ctx.handle, m.ts.data_ptr(), m.qxs.data_ptr(), m.qys.data_ptr(), s.vdf.data_ptr(),
            s.ctx.flux_wall.data_ptr()] + list(extra) + [num.data_ptr(), den.data_ptr(), st]
    return fn(*args)


def test_noalloc_matches_context_scratch_version(cuda):
    s = Solver(small_case(2, 4, 8, 0.3, 0.03, mesh="cavity:12"))
    L = _lib.lib()
    f64 = dict(dtype=torch.float64, device=s.device)
    for call, seed in enumerate((5, 6)):
        _seed(s, seed)
        num0, den0 = torch.zeros(s.ndir, **f64), torch.zeros(s.ndir, **f64)
        num1, den1 = torch.full((s.ndir,), np.nan, **f64), torch.full((s.ndir,), np.nan, **f64)
        _lib.check(_call(L.pbte_transport_residual, s, num0, den0, s.ctx.pbuf.data_ptr()), "reference call")
        torch.cuda.synchronize()
        # this process's own device memory: torch's pool and the library's
        # contexts (not the device-wide free bytes, which other processes move)
        held = (torch.cuda.memory_reserved(), _live_bytes())
        _lib.check(_call(L.pbte_transport_residual_noalloc, s, num1, den1), f"no-alloc call {call}")
        torch.cuda.synchronize()
        assert (torch.cuda.memory_reserved(), _live_bytes()) == held
        a, b = num1.cpu().numpy(), num0.cpu().numpy()
        assert np.abs(a - b).max() <= 1e-12 * np.abs(b).max()
        a, b = den1.cpu().numpy(), den0.cpu().numpy()
        assert np.abs(a - b).max() <= 1e-12 * np.abs(b).max()


def test_noalloc_refuses_periodic_faces(cuda):
    s = Solver(periodic_case(1, 4, 8, 0.5, 0.05))
    f64 = dict(dtype=torch.float64, device=s.device)
    num, den = torch.zeros(s.ndir, **f64), torch.zeros(s.ndir, **f64)
    assert _call(_lib.lib().pbte_transport_residual_noalloc, s, num, den) == -4


def test_noalloc_rejects_cases_beyond_its_scratch(cuda):
    # 130 x 130 squares, P2: 3 * 6 * 33800 = 608400 doubles > 524288
    s = Solver(small_case(2, 2, 4, 0.3, 0.03, mesh="cavity:130"))
    f64 = dict(dtype=torch.float64, device=s.device)
    num, den = torch.zeros(s.ndir, **f64), torch.zeros(s.ndir, **f64)
    assert _call(_lib.lib().pbte_transport_residual_noalloc, s, num, den) == -1
