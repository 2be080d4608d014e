"""Sweep autotuner: times the sweep kernels on a case and keeps the fastest
block shape of the ring sweep (thread groups x threads per group) in the
context.

    python -m pbte_gb300.autotune --grid 64 --deg 2 --npole 8 --nazim 32 --precision fp32

prints one JSON line with the timing of every candidate (CUDA events on the
launching stream, after warm-up) and the choice.  ``--reps`` sets the timed
launches per candidate; ``--only G [--width 64|128]`` times a single shape
(useful under a profiler).
"""
from __future__ import annotations

import argparse
import json

import torch

from .config import square_case
from .solver import Solver

__all__ = ["tune_sweep", "time_sweep"]


def time_sweep(solver, precision: str = "fp32", reps: int = 10, warmup: int = 3) -> float:
    """Average milliseconds of one sweep launch on the solver's case."""
    s = solver
    if precision == "fp32":
        v = torch.zeros(s.vdf.shape, dtype=torch.float32, device=s.device)

        def run():
            s.ctx.sweep_f32((s.mom.ts, s.mom.qxs, s.mom.qys), v, s.ctx.flux_wall)
    else:
        def run():
            s.ctx.sweep(s.mom, s.vdf)
    for _ in range(warmup):
        run()
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    a.record()
    for _ in range(reps):
        run()
    b.record()
    b.synchronize()
    return a.elapsed_time(b) / reps


#: ring sweep block shapes tried by default: (groups, threads per group)
SHAPES = ((2, 64), (3, 64), (4, 64), (6, 64), (8, 64), (2, 128), (3, 128), (4, 128))


def tune_sweep(solver, precision: str = "fp32", candidates=SHAPES, reps: int = 10) -> dict:
    """Time the ring sweep at each block shape, keep the fastest.  A shape is
    ``(groups, threads_per_group)`` or a bare group count (64 threads)."""
    out = {}
    for cand in candidates:
        g, w = (cand, 64) if isinstance(cand, int) else cand
        solver.ctx.set_groups(g, w)
        try:
            out[f"{g}x{w}"] = time_sweep(solver, precision, reps)
        except RuntimeError:
            out[f"{g}x{w}"] = float("inf")
    best = min(out, key=out.get)
    g, w = (int(x) for x in best.split("x"))
    solver.ctx.set_groups(g, w)
    return {"best_groups": g, "best_width": w, "ms": out}


def main(argv=None) -> int:
    ap = argparse.ArgumentParser(description=__doc__)
    ap.add_argument("--grid", type=int, default=64)
    ap.add_argument("--deg", type=int, default=2)
    ap.add_argument("--npole", type=int, default=8)
    ap.add_argument("--nazim", type=int, default=32)
    ap.add_argument("--precision", choices=["fp32", "fp64"], default="fp32")
    ap.add_argument("--mode", choices=["auto", "precomputed", "onthefly"], default="auto")
    ap.add_argument("--reps", type=int, default=10)
    ap.add_argument("--only", type=int, default=0)
    ap.add_argument("--width", type=int, default=64, help="threads per group with --only")
    a = ap.parse_args(argv)
    case = square_case(a.grid, a.deg, a.npole, a.nazim, tau_r=1.0,
                       precision="mixed" if a.precision == "fp32" else "fp64", sweep_mode=a.mode)
    s = Solver(case)
    g = torch.Generator(device="cpu").manual_seed(0)
    for k in ("ts", "qxs", "qys"):
        getattr(s.mom, k).copy_(torch.randn(getattr(s.mom, k).shape, generator=g, dtype=torch.float64))
    cands = ((a.only, a.width),) if a.only else SHAPES
    res = tune_sweep(s, a.precision, cands, a.reps)
    print(json.dumps({"case": vars(a), "schedule": s.ctx.schedule(), "sweep_mode": s.ctx.mode, **res}))
    return 0


if __name__ == "__main__":
    raise SystemExit(main())
