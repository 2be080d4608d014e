#!/usr/bin/env python
"""Benchmark: converged solves/s of the square-cavity DG discrete-ordinates
problem on 8192 triangles, P2, 256 ordinates (the 64 x 64 uniform grid;
west/east isothermal at +0.5/-0.5, north/south diffuse adiabatic).

One step = one converged solve, from a zero state, of one case of the step's
Knudsen sweep (Kn_R in {10, 1, 0.1}, Kn_N = 0.1 Kn_R, cycled), to
<= 1e-8 relative error against the FP64 fixed point, with the
mixed-precision solver (FP32 sweeps, FP64 defect correction, GMRES(30)
inner solve).  Kn_R = 0.01 is not in the GMRES(30) step: restarted GMRES
needs ~6000 sweeps there (measured), the regime GSIS is for.  The timed
region of each step starts with the case's operators and schedule already
on the device.  L2 is flushed (a 512 MB write) before every timed step.

JSON line keys beyond the driver contract: ``roofline`` (the FP32 sweep,
timed live with CUDA events on its stream), ``cpu_baseline`` (the C oracle on
the host cores, one solve), ``e2e`` (the public API from host arrays:
context creation + solve + results to host), ``fp64`` (the plain FP64 GPU
drop-in on the same steps), ``latency_ms`` (p50/p99 of the timed steps),
``batched`` (two copies of each case solved concurrently), ``gsis`` (the FP64
GSIS drop-in at Kn_R = 0.01 with the device trace solve, beside the
per-iteration time with the host trace solve).

``--impl reference`` times the reference algorithm's CPU implementation (the
C oracle, OpenMP over ordinates on all host cores) on the same workload.
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

KN = [10.0, 1.0, 0.1]
GRID, DEG, NPOLE, NAZIM = 64, 2, 8, 32
METRIC = "converged solves/s (<=1e-8 rel err vs FP64, mixed precision)"


def workload_config():
    return {"workload": "square 64x64 grid (8192 tri), DG P2, 256 ordinates (8 polar x 32 azimuth), "
                        "Kn_R cycled over 10/1/0.1, Kn_N=0.1 Kn_R, GMRES(30) mixed FP32/FP64",
            "n_tris": 8192, "ndof": 6, "ndir": 256, "kn_r": KN, "method": "krylov",
            "restart": 30, "tol": 1e-8, "l2": "flushed (512 MB write) before each timed step"}


def make_case(kn, precision="mixed", method="krylov"):
    from pbte_gb300.config import square_case
    return square_case(GRID, DEG, NPOLE, NAZIM, tau_r=kn, tau_n=0.1 * kn, method=method,
                       precision=precision, krylov_restart=30, tol=1e-8, tmax=20000)


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
SWEEP_TRAFFIC = {(8192, 6, 256): 7028480 + 1436672}


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
            "traffic_source": ("ncu dram__bytes_read.sum + dram__bytes_write.sum, one launch, same workload"
                               if traffic is not None else "not captured for this workload")}


def cpu_solve(kn, nthreads, max_seconds=30.0):
    """One solve of the same case with the C oracle on the host cores."""
    from oracle.oracle import Oracle
    from pbte_gb300.discretisation import Discretisation

    disc = Discretisation.build(make_case(kn, precision="fp64"))
    o = Oracle(disc, nthreads=nthreads)
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
    # the timed steps solve exactly the GPU arm's timed sequence of cases
    times = []
    for k in range(args.steps):
        t, r = cpu_solve(KN[k % len(KN)], cores)
        times.append(t)
    total = float(sum(times))
    v = len(times) / total
    line = {"metric": METRIC, "value": round(v, 4), "unit": "solves/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": round(1e3 * total / len(times), 2),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (structured square mesh, seedless)", "impl": "reference",
            "config": {**workload_config(), "method": "GMRES(30) FP64 (C oracle)"},
            "cpu_baseline": {"value": round(v, 4), "unit": "solves/s", "cores": cores, "kind": "port",
                             "sample": f"{len(times)} complete solves, Kn_R sequence "
                                       f"{[KN[k % len(KN)] for k in range(args.steps)]}"},
            "e2e": {"value": round(v, 4), "unit": "solves/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=6)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
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

    def reset(s):
        s.reset()

    def barrier():
        rank_barrier(dist)
        torch.cuda.synchronize(dev)

    def timed(pool, k, check=None):
        kn = KN[k % len(KN)]
        s = pool[kn]
        reset(s)
        flush.fill_(float(k))
        barrier()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record()
        rec = s.run()
        b.record()
        barrier()
        if not rec.converged:
            raise RuntimeError(f"solve at Kn_R={kn} did not converge")
        return a.elapsed_time(b), rec

    for k in range(args.warmup):
        timed(solvers, k)
    launches = 0
    times = []
    mixed_fields = []
    with ClockSampler(local) as clk:
        for k in range(args.steps):
            ms, rec = timed(solvers, k)
            times.append(ms)
            mixed_fields.append((KN[k % len(KN)], rec.temp, rec.qx))
            # per FP32 Arnoldi column: sweep, epilogue (moments, integrals,
            # wall emission), CGS2 (3, the rotation in the last one's tail),
            # next basis vector with the next column's moment sources; one
            # sources launch per inner cycle's first chunk at least; per FP64
            # product: sources, sweep, moments (2), element integrals, wall flux.
            # Not counted: the launches of a ten-column chunk's columns after
            # the cycle's stop, which return at their first instruction
            # (a lower bound, then)
            d = rec.diagnostics
            launches += 6 * d["fp32_sweeps"] + d["outer_steps"] + 6 * d["fp64_sweeps"]
    clocks = clk.summary()
    total = max_over_ranks(float(sum(times)), dist)
    value = replica_throughput(args.steps, total * 1e-3, world)

    # FP64 drop-in on the same steps (reported beside the headline), after
    # one untimed solve of each case (first launches load kernels and
    # capture graphs, as the mixed solver's warm-up steps did)
    for k in range(len(KN)):
        timed(fp64, k)
    t64 = []
    fp64_fields = {}
    for k in range(min(args.steps, len(KN))):
        ms, rec64 = timed(fp64, k)
        t64.append(ms)
        fp64_fields[KN[k % len(KN)]] = (rec64.temp, rec64.qx)

    def rel_l2(a, b):
        return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))

    # every timed mixed solve against the FP64 drop-in's solve of the same
    # case (relative L2 on temperature and heat flux); the bar is 1e-8
    err = max(max(rel_l2(t, fp64_fields[kn][0]), rel_l2(q, fp64_fields[kn][1])) for kn, t, q in mixed_fields)
    if not err <= 1e-8:
        raise RuntimeError(f"mixed-precision solves are {err:.2e} from the FP64 drop-in (bar 1e-8)")
    fp64_rate = len(t64) / (sum(t64) * 1e-3)

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

    # e2e: public API from host arrays -- context creation (H2D of the
    # operators + schedule), solve, fields back to host
    e2e_t, h2d, d2h = [], 0, 0
    from pbte_gb300.sweep import SweepContext
    for k in range(min(args.steps, len(KN))):
        kn = KN[k % len(KN)]
        s = solvers[kn]
        barrier()
        t0 = time.perf_counter()
        s.ctx = SweepContext(s.disc, device=str(dev))
        reset(s)
        rec = s.run()
        out = (rec.temp_dofs, rec.qx_dofs, rec.qy_dofs, rec.temp, rec.qx, rec.qy)
        barrier()
        e2e_t.append(time.perf_counter() - t0)
        h2d = sum(v.nbytes for v in s.ctx._host.values())
        d2h = sum(v.nbytes for v in out)
    e2e = len(e2e_t) / sum(e2e_t)

    # GSIS at Kn_R = 0.01, where GMRES(30) needs ~6000 sweeps: the FP64 GSIS
    # drop-in with the device trace solve (one solve after an untimed one),
    # and the per-iteration time of the same step with the host SuperLU trace
    # solve pybte uses (20 iterations)
    gsis = None
    if rank == 0:
        from pbte_gb300.config import square_case

        def gsis_case(where, tmax=200_000):
            c = square_case(GRID, DEG, NPOLE, NAZIM, tau_r=0.01, tau_n=0.001, accflag=1, tol=1e-8, tmax=tmax)
            c.performance.trace_solver = where
            return c

        g = Solver(gsis_case("device"), device=str(dev))
        g.run()
        g.reset()
        torch.cuda.synchronize(dev)
        t0 = time.perf_counter()
        grec = g.run()
        torch.cuda.synchronize(dev)
        tg = time.perf_counter() - t0
        h = Solver(gsis_case("host", tmax=20), device=str(dev))
        hrec = h.run()
        gsis = {"kn_r": 0.01, "value": round(1.0 / tg, 4), "unit": "solves/s", "converged": bool(grec.converged),
                "iterations": int(grec.iterations), "ms_per_iteration": round(1e3 * tg / grec.iterations, 3),
                "host_trace_ms_per_iteration": round(1e3 * hrec.wall_clock / hrec.iterations, 3),
                "trace_solve": "device nested dissection", "setup_s": round(g.setup_seconds, 2),
                "trace_factor_entries": int(g.acc.solver.factor_entries)}
        del g, h

    peak, kind = read_peaks()
    roof = sweep_roofline(solvers[1.0], peak, kind)
    # the FP32 sweep on the large diffusive square (256 x 256, 131 072
    # triangles, P2, 512 ordinates), where the roofline target is set
    c3 = None
    if rank == 0:
        from pbte_gb300.config import square_case
        t0 = time.perf_counter()
        big = Solver(square_case(256, 2, 8, 64, tau_r=1e-3, tau_n=1e-4, precision="mixed", sweep_mode="onthefly"),
                     device=str(dev))
        c3 = {"workload": "square 256x256 grid (131072 tri), DG P2, 512 ordinates (8 polar x 64 azimuth)",
              "setup_s": round(time.perf_counter() - t0, 2), "roofline": sweep_roofline(big, peak, kind, reps=10)}
        del big
        torch.cuda.empty_cache()
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
                "err_vs_fp64": {"max_rel_l2": float(f"{err:.3e}"), "fields": ["temp", "qx"],
                                "against": "FP64 GPU drop-in solve of the same case (GMRES(30), tol 1e-8)",
                                "bar": 1e-8},
                "fp64": {"value": round(fp64_rate, 4), "unit": "solves/s",
                         "speedup_mixed_over_fp64": round(value / world / fp64_rate, 3),
                         "speedup_batched_mixed_over_fp64": round(batched["value"] / fp64_rate, 3)},
                "batched": batched, "gsis": gsis,
                "e2e": {"value": round(e2e, 4), "unit": "solves/s", "h2d_bytes_per_step": int(h2d),
                        "d2h_bytes_per_step": int(d2h)},
                "roofline": roof, "c3_sweep": c3, "cpu_baseline": cpu, "clocks": clocks,
                "gpu_launches": int(launches)}
        print(json.dumps(line), flush=True)
    if dist is not None:
        dist.barrier()
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
