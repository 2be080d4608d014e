#!/usr/bin/env python
"""Benchmark: converged solves/s of the square-cavity DG discrete-ordinates
problem on 8192 triangles, P2, 256 ordinates (the 64 x 64 uniform grid;
west/east isothermal at +0.5/-0.5, north/south diffuse adiabatic).

One step = one converged solve, from a zero state, of one case of the step's
Knudsen sweep (Kn_R in {10, 1, 0.1, 0.01}, Kn_N = 0.1 Kn_R, cycled) with the
mixed-precision solver (FP32 sweeps, FP64 defect correction): GMRES(30) for
Kn_R >= 0.1, GSIS (inner GMRES(30) on FP32 GSIS products, FP64 trace solve)
at Kn_R = 0.01, where restarted GMRES needs ~6000 sweeps.  Every timed
solve's error against a tight FP64 solve of the same case and method is
measured (``err_vs_fp64``, bar 1e-8).  The timed region of each step starts
with the case's operators and schedule already on the device.  L2 is
flushed (a 512 MB write) before every timed step.

JSON line keys beyond the driver contract: ``fp64`` (the plain FP64 GPU
drop-in, same method per case, on the same steps), ``c2_methods`` (CIS,
GMRES(30) and GSIS, FP64 and mixed, at each Kn_R), ``roofline`` (the FP32
sweep, timed live with CUDA events on its stream), ``c3`` (the large
diffusive square: 131 072 triangles, 512 ordinates, Kn_R = 1e-3, mixed GSIS
against its all-FP64 form, and the FP32 sweep's roofline), ``cpu_baseline``
(the C oracle on the host cores, one solve), ``e2e`` (the public API from
host arrays: operator upload, solve, results to host), ``latency_ms``,
``batched`` (two copies of each case solved concurrently), ``gsis`` (the FP64
GSIS drop-in's iteration, with the device and with the host trace solve),
``batched_c4`` (the first ``--c4`` instances of the batched workload: the
lockstep batch, one sweep launch per DG order for all instances, against the
same solves in sequence, mixed and FP64) and ``serving_c5`` (``--c5``
requests of the served workload at Poisson rate ``--c5-rate``: continuous
batching and one stream per request, against serial FP64 solves).

``--impl reference`` times the reference algorithm's CPU implementation (the
C oracle, OpenMP over ordinates on all host cores) on the same sequence of
cases.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import tempfile
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
sys.path[:0] = [str(ROOT / "ai-driven-numerical-method-exploration-for-multiscale-pbte_gb300"), str(ROOT)]

import numpy as np  # noqa: E402

KN = [10.0, 1.0, 0.1, 0.01]
GRID, DEG, NPOLE, NAZIM = 64, 2, 8, 32
METRIC = "converged solves/s (<=1e-8 rel err vs FP64, mixed precision)"


def method_for(kn):
    """GMRES(30) where it converges in hundreds of sweeps, GSIS below."""
    return "gsis" if kn < 0.05 else "gmres30"


def workload_config():
    return {"workload": "square 64x64 grid (8192 tri), DG P2, 256 ordinates (8 polar x 32 azimuth), "
                        "Kn_R cycled over 10/1/0.1/0.01, Kn_N=0.1 Kn_R; GMRES(30) for Kn_R>=0.1, GSIS at 0.01; "
                        "mixed FP32 sweeps with FP64 defect correction",
            "n_tris": 8192, "ndof": 6, "ndir": 256, "kn_r": KN, "method": {str(k): method_for(k) for k in KN},
            "restart": 30, "tol": 1e-8, "l2": "flushed (512 MB write) before each timed step"}


def make_case(kn, precision="mixed", method=None, tol=1e-8):
    from pbte_gb300.config import square_case
    method = method or method_for(kn)
    kw = dict(tau_r=kn, tau_n=0.1 * kn, precision=precision, krylov_restart=30, tol=tol, tmax=20000)
    if method == "gsis":
        return square_case(GRID, DEG, NPOLE, NAZIM, accflag=1, **kw)
    return square_case(GRID, DEG, NPOLE, NAZIM, method="krylov" if method == "gmres30" else "source", **kw)


def read_peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clock/throttle samples during the timed region."""

    def __init__(self, index=0):
        self.index = index
        self.proc = None
        fd, name = tempfile.mkstemp(prefix="pbte_clocks_", suffix=".csv")
        os.close(fd)
        self.path = Path(name)

    def __enter__(self):
        try:
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), "--query-gpu=clocks.sm,clocks.max.sm,power.draw,"
                 "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
                 "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap",
                 "--format=csv,noheader,nounits", "-lms", "200"], stdout=self.f, stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
        if getattr(self, "f", None) is not None:
            self.f.close()

    def summary(self):
        text = self.path.read_text() if self.path.exists() else ""
        self.path.unlink(missing_ok=True)
        if self.proc is None or not text:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in text.splitlines():
            p = [x.strip() for x in line.split(",")]
            if len(p) < 7:
                continue
            try:
                sm.append(float(p[0]))
                mx.append(float(p[1]))
            except ValueError:
                continue
            for n, v in zip(names, p[3:7]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": float(max(mx)), "reasons": sorted(reasons),
                "samples": len(sm)}


# DRAM bytes of one launch of the FP32 ring sweep (dram__bytes_read.sum +
# dram__bytes_write.sum), by workload (n_tris, ndof, ndir), from the ncu
# captures summarised under profiles/ (sweep_ring_fp32_*); None elsewhere
SWEEP_TRAFFIC = {(8192, 6, 256): 7028480 + 1436672,
                 (32768, 6, 512): 61752064 + 375911680,
                 # the 131 072-triangle sweep, scaled from the 32 768-triangle capture
                 # by the (velocity, element) pairs: its traffic is the distribution's writes
                 (131072, 6, 512): 4 * (61752064 + 375911680)}


def sweep_roofline(solver, peak, peak_kind, reps=20):
    """Average duration of the FP32 sweep kernel on this case (CUDA events on
    its stream) and its algorithmic bytes per launch."""
    import torch

    s = solver
    v32 = torch.zeros(s.vdf.shape, dtype=torch.float32, device=s.device)
    st = torch.cuda.Stream(device=s.device)
    with torch.cuda.stream(st):
        s.mom.ts.normal_()
        s.mom.qxs.normal_()
        s.mom.qys.normal_()
        for _ in range(3):
            s.ctx.sweep_f32((s.mom.ts, s.mom.qxs, s.mom.qys), v32, s.ctx.flux_wall, stream=st)
        a = torch.cuda.Event(enable_timing=True)
        b = torch.cuda.Event(enable_timing=True)
        st.synchronize()
        a.record(st)
        for _ in range(reps):
            s.ctx.sweep_f32((s.mom.ts, s.mom.qxs, s.mom.qys), v32, s.ctx.flux_wall, stream=st)
        b.record(st)
        b.synchronize()
    ms = a.elapsed_time(b) / reps
    nd, nt, ndir = s.ndof, s.n_tris, s.ndir
    algo = (4.0 * ndir * nt * nd                 # write f, every ordinate (FP32)
            + 4.0 * 3 * nt * nd                  # moment sources (FP32)
            + 116.0 * s.ctx.n_classes * nt       # field-major element records, once per direction class
            + 8.0 * s.mesh.n_faces_b * nd)       # wall emission (FP64)
    ach = algo / (ms * 1e-3) / 1e9
    sch = s.ctx.schedule()
    traffic = SWEEP_TRAFFIC.get((nt, nd, ndir))
    return {"bound": "hbm", "achieved": round(ach, 1), "peak": peak, "unit": "GB/s",
            "frac": round(ach / peak, 4), "traffic": traffic,
            "kernel": f"sweep_ring_kernel<float, P{s.case.dg.deg}> (widest level {sch['ring_W']}, "
                      f"{sch['levels']} levels, {sch['unique_dirs']} blocks)",
            "kernel_ms": round(ms, 4), "algorithmic_bytes": int(algo), "peak_source": f"{peak_kind} hbm_gbs",
            "traffic_source": ("not captured for this workload" if traffic is None else
                               "ncu dram__bytes_read.sum + dram__bytes_write.sum of one launch at 32768 triangles, "
                               "x4 (the pairs processed)" if nt == 131072 else
                               "ncu dram__bytes_read.sum + dram__bytes_write.sum, one launch, same workload")}


def cpu_solve(kn, nthreads):
    """One solve of the case with the C oracle on the host cores: seconds and
    the oracle's record.  GMRES(30): the complete solve.  GSIS (Kn_R = 0.01):
    30 iterations timed, scaled to the oracle's full iteration count for this
    case (675, its complete solve recorded in tests/golden/c2_square64_oracle.json:
    one complete solve takes ~9 minutes on the host)."""
    from oracle.oracle import Oracle
    from pbte_gb300.discretisation import Discretisation

    o = Oracle(Discretisation.build(make_case(kn, precision="fp64")), nthreads=nthreads)
    if method_for(kn) == "gsis":
        full = json.loads((ROOT / "tests" / "golden" / "c2_square64_oracle.json").read_text())["gsis_kn0.01"]
        r = o.run_source(tmax=30, gsis=True)
        return r["wall"] / r["iterations"] * full["iterations"], {**r, "iterations": full["iterations"],
                                                                   "sampled_iterations": r["iterations"]}
    t0 = time.perf_counter()
    r = o.run_krylov(tol=1e-8, tmax=20000, max_basis=30)
    return time.perf_counter() - t0, r


def run_reference(args, world, rank):
    if rank != 0:
        return 0
    from oracle import oracle as orc
    orc.build()
    cores = os.cpu_count() or 1
    # warm-up: untimed solves of the cheapest case (the oracle has no caches
    # to fill; this loads the library and pages the code in)
    for _ in range(args.warmup):
        cpu_solve(KN[0], cores)
    # the timed steps are the GPU arm's sequence of cases; each distinct case
    # is solved (or, GSIS, sampled) once and its time counted for every step
    # that repeats it, so the run stays within minutes
    per_case = {}
    times = []
    for k in range(args.steps):
        kn = KN[k % len(KN)]
        if kn not in per_case:
            per_case[kn] = cpu_solve(kn, cores)[0]
        times.append(per_case[kn])
    total = float(sum(times))
    v = len(times) / total
    line = {"metric": METRIC, "value": round(v, 4), "unit": "solves/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": round(1e3 * total / len(times), 2),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (structured square mesh, seedless)", "impl": "reference",
            "config": {**workload_config(), "method": {str(k): method_for(k) + " FP64 (C oracle)" for k in KN}},
            "cpu_baseline": {"value": round(v, 4), "unit": "solves/s", "cores": cores, "kind": "port",
                             "sample": f"Kn_R sequence {[KN[k % len(KN)] for k in range(args.steps)]}; seconds per "
                                       f"case {({str(k): round(t, 2) for k, t in per_case.items()})}: GMRES(30) cases "
                                       "solved completely once, the GSIS case 30 iterations scaled to its 675"},
            "e2e": {"value": round(v, 4), "unit": "solves/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


def rel_l2(a, b):
    a, b = np.asarray(a, dtype=float), np.asarray(b, dtype=float)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def field_error(rec, ref):
    """Relative L2 of the temperature deviation and of the heat-flux vector."""
    return max(rel_l2(rec.temp, ref.temp),
               rel_l2(np.concatenate([rec.qx, rec.qy]), np.concatenate([ref.qx, ref.qy])))


def run_c3(dev, peak, kind):
    """The large diffusive square (256 x 256, 131 072 triangles, P2, 512
    ordinates, Kn_R = 1e-3, Kn_N = 1e-4, adiabatic north/south walls, GSIS):
    the mixed solve (inner GMRES(150) with an FP64 basis on FP32 GSIS
    products, FP64 trace solve and defects) against the same Krylov-accelerated
    defect correction with FP64 products, and the plain FP64 GSIS iteration's
    per-iteration time and progress; plus the FP32 sweep's roofline."""
    import torch
    from pbte_gb300 import Solver
    from pbte_gb300.config import square_case
    from pbte_gb300.mixed import MixedOptions, run_mixed

    t0 = time.perf_counter()
    s = Solver(square_case(256, 2, 8, 64, tau_r=1e-3, tau_n=1e-4, accflag=1, tol=1e-9, tmax=200000,
                           precision="mixed", inner_basis="fp64", krylov_restart=150), device=str(dev))
    setup = time.perf_counter() - t0

    def solve(opts):
        s.reset()
        torch.cuda.synchronize(dev)
        t = time.perf_counter()
        r = run_mixed(s, opts)
        torch.cuda.synchronize(dev)
        return time.perf_counter() - t, r

    solve(MixedOptions())                                       # captures the product and cycle graphs
    tm, rm = solve(MixedOptions())
    fp64_opts = MixedOptions(inner_precision="fp64", inner_rtol=1e-13, refine_tol=1e-13, error_tol=0.0)
    solve(fp64_opts)
    t64, r64 = solve(fp64_opts)
    c = s.case
    keep = c.iteration.tmax
    c.iteration.tmax = 60
    s.reset()
    torch.cuda.synchronize(dev)
    t = time.perf_counter()
    rp = s._run_source("GSIS")
    torch.cuda.synchronize(dev)
    tp = time.perf_counter() - t
    c.iteration.tmax = keep
    out = {"workload": "square 256x256 grid (131072 tri), DG P2, 512 ordinates (8 polar x 64 azimuth), "
                       "Kn_R=1e-3, Kn_N=1e-4, GSIS, mixed solve to an estimated error of 1e-9",
           "setup_s": round(setup, 1),
           "mixed": {"value": round(1.0 / tm, 4), "unit": "solves/s", "seconds": round(tm, 3),
                     "converged": bool(rm.converged), "outer_steps": rm.diagnostics["outer_steps"],
                     "fp32_sweeps": rm.diagnostics["fp32_sweeps"], "fp64_sweeps": rm.diagnostics["fp64_sweeps"],
                     "final_defect": rm.diagnostics["final_defect"], "kappa": rm.diagnostics["kappa"]},
           "fp64": {"value": round(1.0 / t64, 4), "unit": "solves/s", "seconds": round(t64, 3),
                    "converged": bool(r64.converged), "fp64_sweeps": r64.diagnostics["fp64_sweeps"],
                    "form": "the same Krylov-accelerated GSIS defect correction with FP64 products, "
                            "stopped at a defect of 1e-13 (the mixed solve stops on its error estimate 1e-9)"},
           "err_mixed_vs_fp64": float(f"{field_error(rm, r64):.3e}"),
           "speedup_mixed_over_fp64": round(t64 / tm, 3),
           "plain_fp64_gsis": {"ms_per_iteration": round(1e3 * tp / rp.iterations, 3), "iterations": int(rp.iterations),
                               "step_residual": float(f"{rp.residual_history[-1]:.3e}"),
                               "err_vs_fixed_point": float(f"{field_error(rp, r64):.3e}")},
           "sweep_roofline": sweep_roofline(s, peak, kind, reps=10)}
    del s
    torch.cuda.empty_cache()
    return out


def run_c4(dev, count):
    """The batched workload's first ``count`` instances (seed 0: grids 16-128,
    P1-P3, 64-512 ordinates, Kn_R in [1e-3, 10], GSIS, mixed to 1e-8):
    the lockstep batch (one sweep launch per order for all instances'
    products, autotuned block shape) against the same mixed solves one after
    another and against the same solves in FP64 (the Krylov-accelerated GSIS
    defect correction with FP64 products), all with operators resident."""
    import torch
    from pbte_gb300 import Solver
    from pbte_gb300.batch import LockstepBatch, tune_batch_shape
    from pbte_gb300.config import batched_instances
    from pbte_gb300.mixed import MixedOptions, run_mixed

    t0 = time.perf_counter()
    sol = [Solver(c, device=str(dev)) for c in batched_instances(0, count)]
    torch.cuda.synchronize(dev)
    setup = time.perf_counter() - t0
    tune = tune_batch_shape(sol)
    batch = LockstepBatch(sol, shape=tune["choice"])
    batch.run()
    recs = batch.run()
    t_batch = batch.wall_clock
    del batch

    def serial(opts):
        for s in sol:
            s.reset()
            run_mixed(s, opts)
        torch.cuda.synchronize(dev)
        t = time.perf_counter()
        out = []
        for s in sol:
            s.reset()
            out.append(run_mixed(s, opts))
        torch.cuda.synchronize(dev)
        return time.perf_counter() - t, out

    t_serial, _ = serial(MixedOptions())
    t64, r64 = serial(MixedOptions(inner_precision="fp64", inner_rtol=1e-13, refine_tol=1e-13, error_tol=0.0))
    errs = [field_error(a, b) for a, b in zip(recs, r64)]
    err = max(errs)
    worst = int(np.argmax(errs))
    out = {"instances": count, "draw": "config.batched_instances(seed=0), first instances", "setup_s": round(setup, 1),
           "block_shape": list(tune["choice"]), "tune_ms": tune["ms"],
           "lockstep": {"value": round(count / t_batch, 4), "unit": "solves/s", "seconds": round(t_batch, 3),
                        "converged": int(sum(r.converged for r in recs))},
           "serial_mixed": {"value": round(count / t_serial, 4), "unit": "solves/s", "seconds": round(t_serial, 3)},
           "serial_fp64": {"value": round(count / t64, 4), "unit": "solves/s", "seconds": round(t64, 3),
                           "form": "Krylov-accelerated GSIS defect correction with FP64 products, stopped at a "
                                   "defect of 1e-13 (the mixed solves stop on their error estimate 1e-9)"},
           "speedup_lockstep_over_fp64": round(t64 / t_batch, 3),
           "err_vs_fp64": float(f"{err:.3e}"),
           "worst": {"instance": worst, "converged": bool(recs[worst].converged),
                     "fp64_converged": bool(r64[worst].converged),
                     "norm_temp": float(np.linalg.norm(recs[worst].temp)),
                     "fp64_norm_temp": float(np.linalg.norm(r64[worst].temp))}}
    for s in sol:
        s.release()
    del sol
    torch.cuda.empty_cache()
    return out


def run_c5(dev, count, rate):
    """Serving: ``count`` requests of the seed-1 draw (as the batched
    workload), Poisson arrivals at ``rate`` per second, 150 GB budget:
    continuous lockstep batching and one stream per request; latency includes
    each request's set-up (discretisation, operators, trace factorisation)."""
    import torch
    from pbte_gb300 import Solver
    from pbte_gb300.config import batched_instances
    from pbte_gb300.mixed import MixedOptions, run_mixed
    from pbte_gb300.serve import Server

    out = {"requests": count, "rate_per_s": rate, "draw": "config.batched_instances(seed=1)", "budget_gb": 150}
    gaps = np.random.default_rng(1001).exponential(1.0 / rate, size=count)
    for mode in ("lockstep", "streams"):
        srv = Server(device=str(dev), hbm_budget=150e9, slots=8, mode=mode)
        for c, gap in zip(batched_instances(1, count), gaps):
            time.sleep(float(gap))
            srv.submit(c)
        srv.close()
        st = srv.stats()
        out[mode] = {k: (round(v, 3) if isinstance(v, float) else v) for k, v in st.items()}
    # the same requests one after another in FP64, set-up included
    t0 = time.perf_counter()
    lat = []
    for c in batched_instances(1, count):
        t1 = time.perf_counter()
        s = Solver(c, device=str(dev))
        run_mixed(s, MixedOptions(inner_precision="fp64", inner_rtol=1e-12))
        torch.cuda.synchronize(dev)
        s.release()
        lat.append(time.perf_counter() - t1)
    span = time.perf_counter() - t0
    out["serial_fp64"] = {"solves_per_s": round(count / span, 3), "p50_ms": round(float(np.percentile(lat, 50)) * 1e3, 1),
                          "p99_ms": round(float(np.percentile(lat, 99)) * 1e3, 1),
                          "form": "Krylov-accelerated GSIS with FP64 products, set-up included"}
    torch.cuda.empty_cache()
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=8)
    ap.add_argument("--warmup", type=int, default=4)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-c3", action="store_true", help="skip the 131 072-triangle solve (~3 minutes)")
    ap.add_argument("--no-methods", action="store_true", help="skip the CIS/GMRES/GSIS method table")
    ap.add_argument("--c4", type=int, default=16, help="instances of the batched workload (0: skip; 64: all)")
    ap.add_argument("--c5", type=int, default=16, help="requests of the served workload (0: skip)")
    ap.add_argument("--c5-rate", type=float, default=1.0, help="Poisson arrivals per second")
    args = ap.parse_args()
    args.warmup = max(3, args.warmup)

    from pbte_gb300.replicas import barrier as rank_barrier, max_over_ranks, rank_info, replica_throughput
    info = rank_info()
    world, rank, local = info.world, info.rank, info.local
    if args.impl == "reference":
        return run_reference(args, world, rank)

    import torch
    dist = None
    if world > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    dev = torch.device(f"cuda:{local}")
    torch.cuda.set_device(dev)
    from pbte_gb300 import Solver, _lib
    _lib.lib()

    # cases resident on the device before timing (replicas: every rank its own copy)
    solvers = {kn: Solver(make_case(kn), device=str(dev)) for kn in KN}
    fp64 = {kn: Solver(make_case(kn, precision="fp64"), device=str(dev)) for kn in KN}
    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)

    def barrier():
        rank_barrier(dist)
        torch.cuda.synchronize(dev)

    def timed(s, k, check=True):
        s.reset()
        flush.fill_(float(k))
        barrier()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record()
        rec = s.run()
        b.record()
        barrier()
        if check and not rec.converged:
            raise RuntimeError(f"solve of {s.case.flow.tau_r} ({s.precision}) did not converge")
        return a.elapsed_time(b), rec

    # the FP64 fixed point of every case, to 1e-12 (same method, so GSIS is
    # measured against the GSIS fixed point): what the errors are taken against
    tight = {}
    for kn, s in fp64.items():
        s.case.iteration.tol = 1e-12
        s.reset()
        tight[kn] = s.run()
        s.case.iteration.tol = 1e-8

    for k in range(args.warmup):
        timed(solvers[KN[k % len(KN)]], k)
    launches = 0
    times = []
    errs = []
    with ClockSampler(local) as clk:
        for k in range(args.steps):
            kn = KN[k % len(KN)]
            ms, rec = timed(solvers[kn], k)
            times.append(ms)
            errs.append(field_error(rec, tight[kn]))
            # per FP32 product: the sweep, its epilogue (GMRES) or the GSIS
            # chain (hot source, wall traces, right-hand side, ~20 trace-solve
            # heights, recovery, correction), CGS2 (3, the rotation in the
            # last), next basis; per FP64 product: sources, sweep, moments or
            # the GSIS chain, emission.  Not counted: launches of a ten-column
            # chunk after its cycle's stop, which return at their first
            # instruction (a lower bound, then)
            d = rec.diagnostics
            per32, per64 = (6, 6) if method_for(kn) == "gmres30" else (34, 32)
            launches += per32 * d["fp32_sweeps"] + d["outer_steps"] + per64 * d["fp64_sweeps"]
    clocks = clk.summary()
    total = max_over_ranks(float(sum(times)), dist)
    value = replica_throughput(args.steps, total * 1e-3, world)
    err = max(errs)
    if not err <= 1e-8:
        raise RuntimeError(f"mixed-precision solves are {err:.2e} from the FP64 fixed point (bar 1e-8)")

    # FP64 drop-in on the same steps (one untimed solve of each case first:
    # first launches load kernels and capture graphs, as the mixed solver's
    # warm-up steps did)
    for k in range(len(KN)):
        timed(fp64[KN[k]], k)
    t64 = []
    err64 = {}
    for k in range(args.steps):
        kn = KN[k % len(KN)]
        ms, rec64 = timed(fp64[kn], k)
        t64.append(ms)
        err64[kn] = field_error(rec64, tight[kn])
    fp64_rate = len(t64) / (sum(t64) * 1e-3)
    per_case = {str(kn): {"mixed_ms": round(float(np.mean([t for j, t in enumerate(times)
                                                            if KN[j % len(KN)] == kn])), 3),
                          "fp64_ms": round(float(np.mean([t for j, t in enumerate(t64)
                                                          if KN[j % len(KN)] == kn])), 3),
                          "method": method_for(kn)} for kn in KN}

    # the C2 method table: CIS, GMRES(30) and GSIS, FP64 and mixed, at every
    # Kn_R (one warm solve each; CIS at Kn_R = 0.01 needs tens of thousands of
    # sweeps and is left out); errors against the tight FP64 solve of the
    # same fixed point (CIS and GMRES share one, GSIS has its own)
    methods = None
    if rank == 0 and not args.no_methods:
        methods = {}
        for kn in KN:
            row = {}
            gm_ref = tight[kn] if method_for(kn) == "gmres30" else None
            if gm_ref is None:
                r = Solver(make_case(kn, precision="fp64", method="gmres30", tol=1e-12), device=str(dev))
                gm_ref = r.run()
                del r
            for meth in ("cis", "gmres30", "gsis"):
                if meth == "cis" and kn < 0.05:
                    continue
                ref = tight[kn] if meth == "gsis" and method_for(kn) == "gsis" else None
                if meth == "gsis" and ref is None:
                    r = Solver(make_case(kn, precision="fp64", method="gsis", tol=1e-12), device=str(dev))
                    ref = r.run()
                    del r
                if meth != "gsis":
                    ref = gm_ref
                for prec in ("fp64", "mixed"):
                    sv = (fp64 if prec == "fp64" else solvers)[kn] if meth == method_for(kn) else \
                        Solver(make_case(kn, precision=prec, method=meth), device=str(dev))
                    timed(sv, 0, check=False)
                    ms, rec = timed(sv, 1, check=False)
                    row[f"{meth}_{prec}"] = {"ms": round(ms, 3), "iterations": int(rec.iterations),
                                             "converged": bool(rec.converged),
                                             "err": float(f"{field_error(rec, ref):.3e}")}
            methods[str(kn)] = row
        torch.cuda.empty_cache()

    # batched: two copies of each Kn case solved concurrently (one stream and
    # host thread per solve, pbte_gb300.batch); same results as alone
    from pbte_gb300.batch import BatchSolver
    batch = BatchSolver(list(solvers.values()) + [Solver(make_case(kn), device=str(dev)) for kn in KN])
    batch.prepare()
    bt = []
    for k in range(2):
        flush.fill_(float(k))
        barrier()
        recs = batch.run()
        if not all(r.converged for r in recs):
            raise RuntimeError("a batched solve did not converge")
        bt.append(batch.wall_clock)
    batched = {"value": round(len(batch.solvers) * len(bt) / sum(bt), 4), "unit": "solves/s",
               "solves_per_batch": len(batch.solvers), "ms_per_batch": round(1e3 * sum(bt) / len(bt), 3)}
    for s in solvers.values():
        s.ctx.set_groups(0, 0)
    del batch

    # e2e: the public API from host arrays -- the case's operators uploaded
    # (context creation; for GSIS also the HDG operators and the trace
    # factorisation), the solve, fields back to host
    e2e_t, h2d, d2h = [], 0, 0
    from pbte_gb300.gsis import GSIS
    from pbte_gb300.sweep import SweepContext
    for k in range(len(KN)):
        kn = KN[k]
        s = solvers[kn]
        barrier()
        t0 = time.perf_counter()
        s.ctx = SweepContext(s.disc, device=str(dev))
        if s.acc is not None:
            s.acc = GSIS(s)
        s.reset()
        rec = s.run()
        out = (rec.temp_dofs, rec.qx_dofs, rec.qy_dofs, rec.temp, rec.qx, rec.qy)
        barrier()
        e2e_t.append(time.perf_counter() - t0)
        h2d += sum(v.nbytes for v in s.ctx._host.values()) + (s.acc.h2d_bytes if s.acc is not None else 0)
        d2h += sum(v.nbytes for v in out)
    e2e = len(e2e_t) / sum(e2e_t)

    # the FP64 GSIS drop-in's iteration at Kn_R = 0.01 with the device trace
    # solve, and with the host SuperLU trace solve pybte uses (20 iterations)
    gsis = None
    if rank == 0:
        g = fp64[0.01]
        hc = make_case(0.01, precision="fp64")
        hc.performance.trace_solver = "host"
        hc.iteration.tmax = 20
        h = Solver(hc, device=str(dev))
        hrec = h.run()
        g.reset()
        grec = g.run()
        gsis = {"kn_r": 0.01, "iterations": int(grec.iterations),
                "ms_per_iteration": round(1e3 * grec.wall_clock / grec.iterations, 3),
                "host_trace_ms_per_iteration": round(1e3 * hrec.wall_clock / hrec.iterations, 3),
                "trace_solve": "device nested dissection", "setup_s": round(g.setup_seconds, 2),
                "trace_factor_entries": int(g.acc.solver.factor_entries)}
        del h

    peak, kind = read_peaks()
    roof = sweep_roofline(solvers[1.0], peak, kind)
    c3 = c4 = c5 = None
    if rank == 0:
        del solvers, fp64
        torch.cuda.empty_cache()
        if not args.no_c3:
            c3 = run_c3(dev, peak, kind)
        if args.c4:
            c4 = run_c4(dev, args.c4)
        if args.c5:
            c5 = run_c5(dev, args.c5, args.c5_rate)
    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        from oracle import oracle as orc
        orc.build()
        cores = os.cpu_count() or 1
        t, r = cpu_solve(1.0, cores)
        cpu = {"value": round(1.0 / t, 4), "unit": "solves/s", "cores": cores, "kind": "port",
               "sample": f"1 complete FP64 GMRES(30) solve at Kn_R=1 ({r['iterations']} sweeps, {t:.1f} s)"}
    if rank == 0:
        lat = np.array(times)
        line = {"metric": METRIC, "value": round(value, 4), "unit": "solves/s", "n_gpus": world,
                "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(total / args.steps, 3),
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64",
                "data": "synthetic (structured square mesh)",
                "config": {**workload_config(), "parallelism": f"replicas x{world}"},
                "latency_ms": {"p50": round(float(np.percentile(lat, 50)), 3),
                               "p99": round(float(np.percentile(lat, 99)), 3)},
                "err_vs_fp64": {"max_rel_l2": float(f"{err:.3e}"), "fields": ["temp", "(qx, qy)"],
                                "against": "FP64 GPU solve of the same case and method to 1e-12", "bar": 1e-8},
                "fp64": {"value": round(fp64_rate, 4), "unit": "solves/s",
                         "speedup_mixed_over_fp64": round(value / world / fp64_rate, 3),
                         "speedup_batched_mixed_over_fp64": round(batched["value"] / fp64_rate, 3),
                         "err_vs_fixed_point": {str(k): float(f"{v:.3e}") for k, v in err64.items()},
                         "note": "the drop-in stops on pybte's rule at tol 1e-8"},
                "per_case": per_case, "c2_methods": methods, "batched": batched, "gsis": gsis,
                "e2e": {"value": round(e2e, 4), "unit": "solves/s", "h2d_bytes_per_step": int(h2d / len(KN)),
                        "d2h_bytes_per_step": int(d2h / len(KN))},
                "roofline": roof, "c3": c3, "batched_c4": c4, "serving_c5": c5, "cpu_baseline": cpu,
                "clocks": clocks,
                "gpu_launches": int(launches)}
        print(json.dumps(line), flush=True)
    if dist is not None:
        dist.barrier()
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
