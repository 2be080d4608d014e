"""Command line, as pybte's (``pybte/__main__.py``):

    python -m pbte_gb300 run  case.json [--tmax N] [--tol T] [--out DIR] [--no-output] [--quiet]
    python -m pbte_gb300 info case.json
    python -m pbte_gb300 square N DEG NPOLE NAZIM KN_R [--method source|krylov|gsis]
                                [--precision fp64|mixed] [--repeat R]

A case file is pybte's case dictionary as JSON (``Case.from_dict``; pybte
reads the same dictionary from YAML).  ``square`` solves the benchmark
square (west/east isothermal +0.5/-0.5, north/south diffuse adiabatic,
Kn_N = 0.1 Kn_R), ``--repeat`` times from a zero state.  ``run`` exits 0
when the solve converged, 1 otherwise.
"""
from __future__ import annotations

import argparse
import json
import sys
import time
from pathlib import Path


def _cmd_run(args) -> int:
    from .config import Case
    from .solver import Solver

    path = Path(args.case)
    case = Case.from_dict(json.loads(path.read_text()), basedir=str(path.parent))
    if args.tmax is not None:
        case.iteration.tmax = args.tmax
    if args.tol is not None:
        case.iteration.tol = args.tol
    if args.out is not None:
        case.output.dir = args.out
    if args.no_output:
        case.output.field = case.output.run_record = case.output.runtime_log = False
    solver = Solver(case)
    if not args.quiet:
        print(f"pbte_gb300: {case.mesh_path()}  N_TRIS={solver.n_tris} N_FCS={solver.mesh.n_faces}  "
              f"DEG={case.dg.deg}  NPOLE={case.velmesh.npole} NAZIM={case.velmesh.nazim}")
        print(f"       setup {solver.setup_seconds:.2f}s, sweep mode {solver.ctx.mode}, "
              f"precision {case.performance.precision}")
    rec = solver.run(progress_every=args.progress)
    written = solver.write_outputs(rec)
    if not args.quiet:
        print(f"  iterations      {rec.iterations}{'  (converged)' if rec.converged else '  (TMAX reached)'}")
        print(f"  residual        {rec.final_residual:.6e}")
        print(f"  mass (int T dA) {rec.mass:.12f}")
        print(f"  sweeps          {rec.sweep_count}")
        print(f"  wall clock      {rec.wall_clock:.3f} s")
        for k, v in written.items():
            print(f"  wrote {k:12s} {v}")
    return 0 if rec.converged else 1


def _cmd_info(args) -> int:
    from .config import Case
    from .discretisation import Discretisation

    path = Path(args.case)
    case = Case.from_dict(json.loads(path.read_text()), basedir=str(path.parent))
    d = Discretisation.build(case)
    print(f"mesh            {case.mesh_path()}")
    print(f"  triangles     {d.mesh.n_tris}")
    print(f"  faces         {d.mesh.n_faces} ({d.mesh.n_faces_b} boundary)")
    print(f"  hmin          {d.mesh.hmin:.6e}")
    print(f"discretisation  DEG={case.dg.deg} NDOF_TRI={case.ndof_tri} NDOF_FC={case.ndof_fc}")
    print(f"  directions    {d.ndir}")
    for b in case.boundaries:
        print(f"  {b.name:8s} phyid={b.phyid:3d} type={b.type:16s} T={b.temp:g}")
    print(f"config hash     {case.config_hash}")
    return 0


def _cmd_square(args) -> int:
    import torch

    from .config import square_case
    from .solver import Solver

    gsis = args.method == "gsis"
    case = square_case(args.n, args.deg, args.npole, args.nazim, tau_r=args.kn,
                       method="source" if gsis else args.method, accflag=1 if gsis else 0,
                       precision=args.precision, krylov_restart=30 if args.method == "krylov" else None,
                       tol=args.tol, tmax=args.tmax)
    s = Solver(case)
    ok = True
    for r in range(args.repeat):
        s.reset()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        rec = s.run()
        torch.cuda.synchronize()
        ok = ok and rec.converged
        print(f"solve {r}: {rec.iterations} iterations, converged {rec.converged}, "
              f"{1e3 * (time.perf_counter() - t0):.2f} ms, mass {rec.mass:.12e}", flush=True)
    return 0 if ok else 1


def main(argv=None) -> int:
    p = argparse.ArgumentParser(prog="pbte_gb300", description=__doc__,
                                formatter_class=argparse.RawDescriptionHelpFormatter)
    sub = p.add_subparsers(dest="cmd", required=True)
    r = sub.add_parser("run", help="solve a case")
    r.add_argument("case")
    r.add_argument("--tmax", type=int, default=None)
    r.add_argument("--tol", type=float, default=None)
    r.add_argument("--out", default=None, help="override output.dir")
    r.add_argument("--progress", type=int, default=0)
    r.add_argument("--no-output", action="store_true")
    r.add_argument("--quiet", action="store_true")
    r.set_defaults(fn=_cmd_run)
    i = sub.add_parser("info", help="describe a case without solving it")
    i.add_argument("case")
    i.set_defaults(fn=_cmd_info)
    q = sub.add_parser("square", help="solve the benchmark square")
    for name in ("n", "deg", "npole", "nazim"):
        q.add_argument(name, type=int)
    q.add_argument("kn", type=float)
    q.add_argument("--method", default="krylov", choices=["source", "krylov", "gsis"])
    q.add_argument("--precision", default="mixed", choices=["fp64", "mixed"])
    q.add_argument("--tol", type=float, default=1e-8)
    q.add_argument("--tmax", type=int, default=200_000)
    q.add_argument("--repeat", type=int, default=1)
    q.set_defaults(fn=_cmd_square)
    args = p.parse_args(argv)
    return args.fn(args)


if __name__ == "__main__":
    sys.exit(main())
