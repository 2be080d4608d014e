"""Mixed precision: FP32 sweeps inside an FP64 defect-correction loop.

The outer problem is the fixed point ``u = F(u) = T u + g`` of source
iteration (``u``: the moments, plus the wall emission with adiabatic walls),
or, for a case with the GSIS acceleration, of the GSIS iteration (``F``: a
sweep followed by the acceleration step, :class:`pbte_gb300.gsis.GsisFixedPoint`;
the HDG trace solve stays FP64 in both of its forms).  Each outer step

1. evaluates the FP64 defect ``r = F64(u) - u`` with one FP64 sweep, moments
   and emission (exactly one CIS or GSIS step of the FP64 solver);
2. solves the correction equation ``(I - T) d = r`` approximately with
   FP32 sweeps of the homogeneous problem (no wall sources): either source
   iteration (``method = "source"``) or GMRES (``method = "krylov"``), both
   with FP64 vectors;
3. updates ``u += d``.

Because ``r`` is formed in FP64, the FP32 round-off of the inner sweeps only
limits how much each outer step gains (about 1e-5..1e-6 per step), not the
final accuracy.  The error of ``u`` against the fixed point is
``(I - T)^-1 r``.  ``kappa``, the estimate of that amplification, is the
largest of the corrections' ``||d|| / ||r||`` (each ``d`` solved
``(I - T) d = r`` for an earlier defect) and of ``1 / sigma_min`` of the
inner GMRES cycles' Hessenberg matrices (``(I - T)^-1`` on the Krylov
spaces, which hold the slow modes that dominate the error); the loop stops
when ``kappa * ||r|| <= error_tol * ||F64(u)||`` (or ``||r|| <= refine_tol
* ||F64(u)||``).  A well-conditioned case stops at a larger defect than an
ill-conditioned, diffusive one.  The reported state is ``F64(u)``, an FP64
sweep of the converged state.
"""
from __future__ import annotations

import time

import numpy as np
import torch

from .device import sync
from .krylov import ArnoldiGraphs, FixedPointOperator, amplification, basis_cap, cached, gmres

__all__ = ["run_mixed", "MixedOptions", "refined"]


class MixedOptions:
    #: stop when the estimated error kappa * ||r|| / ||F64(u)|| is below
    #: this, a tenth of the benchmarks' 1e-8 bar (kappa: the estimate of
    #: ||(I - T)^-1|| above.  On the 256 x 256 square at Kn_R 1e-3 a defect
    #: of 5e-12 left an error of 1.0e-8 where the corrections alone gave
    #: kappa 129, a defect of 1e-11 an error of 1.1e-8: ||(I - T)^-1|| is
    #: ~1e3 there, which only the Hessenberg estimate sees early) ...
    error_tol = 1e-9
    #: ... or when the defect ||r|| / ||F64(u)|| itself is below this
    refine_tol = 1e-13
    #: kappa before any correction has been solved (a restart from a
    #: converged state stops at once on a defect below error_tol / kappa0)
    kappa0 = 100.0
    inner_rtol = 1e-6       # inner relative accuracy per outer step (FP32 limits it to ~1e-6)
    max_outer = 200         # outer steps (one inner GMRES cycle each by default)
    max_inner = 200_000
    #: inner GMRES restart cycles per outer step before handing back to the
    #: FP64 defect correction.  One cycle per outer step measured fastest on
    #: the square cavity (Kn_R 10/1/0.1: 21/90/360 FP32 sweeps against
    #: 21/82/600 with four cycles): a fresh FP64 defect restarts GMRES where
    #: its early, fast convergence is, and FP32 round-off cannot stall it.
    inner_budget_restarts = 1
    #: "fp32": the inner products are FP32 sweeps (the mixed-precision
    #: solve); "fp64": FP64 products of the same map (T u = F64(u) - F64(0)),
    #: the all-FP64 form of the same Krylov-accelerated defect correction, the
    #: FP64 comparator where the plain FP64 iteration is too slow to run to
    #: convergence (GSIS with adiabatic walls on large meshes)
    inner_precision = "fp32"

    def __init__(self, **kw):
        for k, v in kw.items():
            if not hasattr(type(self), k):
                raise TypeError(f"unknown mixed-precision option {k!r}")
            setattr(self, k, v)


def refined(rn: float, fn: float, kappa: float | None, opts: MixedOptions) -> bool:
    """The outer stop rule: the defect ``rn`` (of ``||F64(u)|| = fn``) is
    small enough for the error estimate ``kappa * rn`` (``kappa`` None: no
    correction solved yet, ``opts.kappa0``) or on its own."""
    k = opts.kappa0 if kappa is None else kappa
    return rn <= opts.refine_tol * fn or k * rn <= opts.error_tol * fn


def run_mixed(solver, opts: MixedOptions | None = None):
    opts = opts or MixedOptions()
    c = solver.case
    gsis = solver.acc is not None
    if gsis:
        # the fixed point of the GSIS iteration (not CIS's: GSIS converges to
        # its own discrete fixed point), refined around FP32 GSIS products;
        # the inner solve is GMRES, which does not stall on the slow wall
        # modes that plain GSIS iteration meets with adiabatic walls
        from .gsis import GsisFixedPoint
        method = "krylov"
        op64 = cached(solver, "gsis64", lambda: GsisFixedPoint(solver, "fp64"))
        op32 = cached(solver, "gsis32h", lambda: GsisFixedPoint(solver, "fp32", homogeneous=True))
    else:
        method = "krylov" if c.scheme.method == "krylov" else "source"
        op64 = cached(solver, "fp64", lambda: FixedPointOperator(solver, "fp64"))
        op32 = cached(solver, "fp32h",
                      lambda: FixedPointOperator(solver, "fp32", homogeneous=True, integrals=False))
    inner64 = opts.inner_precision == "fp64"
    g0 = None
    if inner64:
        method = "krylov"
        if gsis:
            op32 = cached(solver, "gsis64i", lambda: GsisFixedPoint(solver, "fp64"))
        else:
            op32 = cached(solver, "fp64i", lambda: FixedPointOperator(solver, "fp64"))
    op64.sweeps = op32.sweeps = 0
    n = op64.n
    dev = solver.device
    restarted = bool(getattr(solver, "restart_info", {}).get("enabled"))
    u = op64.state() if restarted else torch.zeros(n, dtype=torch.float64, device=dev)
    ar32 = None
    history = []
    inner_sweeps = 0
    kappa = None           # the largest ||d|| / ||r|| of the corrections
    converged = False
    sync(dev)
    t0 = time.perf_counter()
    if inner64:
        g0 = op32.apply(torch.zeros(n, dtype=torch.float64, device=dev))   # F64(0): the affine part
    fu = op64.apply(u)
    for outer in range(opts.max_outer):
        r = fu - u
        rn = float(torch.linalg.vector_norm(r).item())
        fn = float(torch.linalg.vector_norm(fu).item()) or 1.0
        history.append(rn / fn)
        if refined(rn, fn, kappa, opts):
            converged = True
            break
        if op64.sweeps + inner_sweeps >= c.iteration.tmax:
            break
        if method == "source":
            d = r.clone()
            for _ in range(opts.max_inner):
                dn = op32.apply(d) + r
                inner_sweeps += 1
                step = float(torch.linalg.vector_norm(dn - d).item())
                d = dn
                if step <= opts.inner_rtol * float(torch.linalg.vector_norm(d).item()):
                    break
        else:
            cap = basis_cap(c, n)
            if ar32 is None:
                bdt = torch.float32 if c.performance.inner_basis == "fp32" and not inner64 else torch.float64
                ar32 = cached(solver, ("arnoldi_inner", cap, bdt, inner64),
                              lambda: ArnoldiGraphs(op32, g0, cap, dtype=bdt))
                if inner64:
                    ar32.set_g(g0)
            before = op32.sweeps
            cycles = []
            if inner64:
                mv = lambda v: v - (op32.apply(v) - g0)   # noqa: E731
            else:
                mv = lambda v: v - op32.apply(v)          # noqa: E731
            d, _, _ = gmres(mv, r, ar32, tol_abs=opts.inner_rtol * rn,
                            maxiter=min(opts.max_inner, opts.inner_budget_restarts * cap),
                            on_cycle=lambda R: cycles.append(amplification(R)))
            inner_sweeps += op32.sweeps - before
            if cycles:
                kappa = max(cycles) if kappa is None else max([kappa] + cycles)
        if rn > 0:
            amp = float(torch.linalg.vector_norm(d).item()) / rn
            kappa = amp if kappa is None else max(kappa, amp)
        u = u + d
        fu = op64.apply(u)
    op64.publish()
    sync(dev)
    wall = time.perf_counter() - t0
    sweeps64 = op64.sweeps
    solver.ctx.sweep_count += sweeps64 + inner_sweeps
    rec = solver._record(sweeps64 + inner_sweeps, converged, np.array(history),
                         np.full(len(history), solver.mom.mass), wall,
                         "GSIS" if gsis else ("KRYLOV" if method == "krylov" else "CIS"),
                         extra={"fp64_sweeps": sweeps64 + (inner_sweeps if inner64 else 0),
                                "fp32_sweeps": 0 if inner64 else inner_sweeps,
                                "inner_precision": opts.inner_precision,
                                "outer_steps": len(history), "final_defect": history[-1],
                                "kappa": kappa})
    return rec
