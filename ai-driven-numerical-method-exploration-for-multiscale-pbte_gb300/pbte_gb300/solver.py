"""Outer iterations on the GPU behind pybte's ``Solver`` interface.

``Solver(case).run()`` returns a :class:`RunRecord`, as pybte's does
(``pybte/driver.py:43-254``):

* ``scheme.method = "source"``, ``accflag = 0`` -- CIS (``driver.py:170-215``).
  One outer iteration is [wall emission] -> sweep -> moments -> step residual
  -> stopping rule, all on the device; a block of iterations is captured once
  as a CUDA graph and replayed, with a device-side stop flag so the run ends
  on exactly the iteration where the residual first drops under ``tol``.
* ``accflag = 1`` -- GSIS (:mod:`pbte_gb300.gsis`).
* ``scheme.method = "krylov"`` -- GMRES on the outer fixed point
  (``pybte/krylov.py:257-363``), basis on the device, one sweep per product.

``performance.precision = "mixed"`` runs the same scheme with FP32 sweeps
inside an FP64 defect-correction loop (:mod:`pbte_gb300.mixed`).

Restart files (``VDFP{deg}T{n_tris}NP{npole}NA{nazim}.out``, the Fortran's
``VDF(NDOF, N_TRIS, NPOLE, NAZIM)`` as raw little-endian doubles) are read
at construction and written by :meth:`Solver.save_restart`
(``pybte/driver.py:99-141``); :meth:`Solver.write_outputs` writes the run
record, ``RunTime.txt`` and the sampled fields (``driver.py:256-291``).
"""
from __future__ import annotations

import hashlib
import json
import platform
import sys
import time
import warnings
from dataclasses import dataclass, field, fields
from pathlib import Path

import numpy as np
import torch

from . import _lib
from .config import Case
from .device import bury, device_lock, empty_graveyard, sync
from .discretisation import Discretisation
from .sweep import HostReadable, Moments, SweepContext

__all__ = ["Solver", "RunRecord"]


def _empty(*shape):
    return field(default_factory=lambda: np.zeros(shape))


@dataclass
class RunRecord:
    """pybte's machine-readable run record (``pybte/io_output.py:30-164``):
    the same fields, helpers and JSON / npz writers, plus ``precision``;
    arrays are host numpy."""
    iterations: int = 0
    converged: bool = False
    residual_history: np.ndarray = _empty(0)
    residual_true: np.ndarray | None = None
    mass_history: np.ndarray = _empty(0)
    temp: np.ndarray = _empty(0)
    qx: np.ndarray = _empty(0)
    qy: np.ndarray = _empty(0)
    temp_dofs: np.ndarray = _empty(0, 0)
    qx_dofs: np.ndarray = _empty(0, 0)
    qy_dofs: np.ndarray = _empty(0, 0)
    sweep_count: int = 0
    factorisation_count: int = 0
    wall_clock: float = 0.0
    setup_wall_clock: float = 0.0
    config_hash: str = ""
    scheme: str = "CIS"
    acc_variant: str | None = None
    tol: float = 0.0
    tmax: int = 0
    tau_r: float = 0.0
    tau_n: float = 0.0
    tau_c: float = 0.0
    deg: int = 0
    npole: int = 0
    nazim: int = 0
    n_tris: int = 0
    n_faces: int = 0
    mesh_file: str = ""
    restart: dict = field(default_factory=dict)
    environment: dict = field(default_factory=dict)
    diagnostics: dict = field(default_factory=dict)
    precision: str = "fp64"

    @property
    def final_residual(self) -> float:
        h = np.asarray(self.residual_history)
        return float(h[-1]) if h.size else float("nan")

    @property
    def mass(self) -> float:
        t = np.asarray(self.temp)
        return float(np.sum(t)) if t.size else float("nan")

    @property
    def contraction(self) -> float:
        """Geometric decay rate of the second half of the residual history
        (``io_output.py:76-94``): ``(r_last / r_first) ** (1 / (n - 1))`` over
        its finite positive entries, or ``nan`` if there are fewer than 8
        residuals, fewer than 4 usable ones, no decay, or a rate outside
        (0, 1)."""
        h = np.asarray(self.residual_history, dtype=float)
        if h.size < 8:
            return float("nan")
        tail = h[max(1, h.size // 2):]
        tail = tail[np.isfinite(tail) & (tail > 0)]
        if tail.size < 4 or not tail[-1] < tail[0]:
            return float("nan")
        rho = (tail[-1] / tail[0]) ** (1.0 / (tail.size - 1))
        return float(rho) if 0.0 < rho < 1.0 else float("nan")

    @property
    def error_estimate(self) -> float:
        """Remaining distance to the fixed point of a linearly converging
        iteration, ``r rho / (1 - rho)`` (``io_output.py:96-112``)."""
        rho = self.contraction
        return float(self.final_residual * rho / (1.0 - rho)) if np.isfinite(rho) else float("nan")

    def to_dict(self, include_fields: bool = True) -> dict:
        """JSON-ready dict; ``include_fields=False`` drops the 2-D arrays
        (``io_output.py:114-126``)."""
        d = {}
        for f in fields(self):
            v = getattr(self, f.name)
            if isinstance(v, np.ndarray):
                v = None if (not include_fields and v.ndim > 1) else v.tolist()
            elif isinstance(v, (dict, list)):
                v = json.loads(json.dumps(v, default=_jsonable))
            d[f.name] = v
        d.update(final_residual=self.final_residual, mass=self.mass, contraction=self.contraction,
                 error_estimate=self.error_estimate)
        return d

    def to_json(self, path, include_fields: bool = True) -> Path:
        path = Path(path)
        path.parent.mkdir(parents=True, exist_ok=True)
        path.write_text(json.dumps(self.to_dict(include_fields), indent=2))
        return path

    def to_npz(self, path) -> Path:
        """Every array field plus ``meta``, the field-less dict as JSON
        (``io_output.py:134-141``)."""
        path = Path(path)
        path.parent.mkdir(parents=True, exist_ok=True)
        payload = {f.name: getattr(self, f.name) for f in fields(self)
                   if isinstance(getattr(self, f.name), np.ndarray)}
        payload["meta"] = np.array(json.dumps(self.to_dict(include_fields=False)))
        np.savez_compressed(path, **payload)
        return path

    @staticmethod
    def environment_fingerprint() -> dict:
        import scipy

        return {"python": sys.version.split()[0], "numpy": np.__version__, "scipy": scipy.__version__,
                "numba": None, "torch": torch.__version__, "cuda": torch.version.cuda,
                "platform": platform.platform(), "machine": platform.machine(),
                "device": torch.cuda.get_device_name() if torch.cuda.is_available() else None}


def _jsonable(v):
    if isinstance(v, np.generic):
        return v.item()
    if isinstance(v, np.ndarray):
        return v.tolist()
    return str(v)


class Solver:
    """Set up a case on the GPU and run it to convergence."""

    def __init__(self, case: Case, device: str = "cuda", graph_block: int = 32,
                 discretisation: Discretisation | None = None):
        t0 = time.perf_counter()
        self.case = case
        self.device = torch.device(device)
        self.disc = discretisation if discretisation is not None else Discretisation.build(case)
        self.mesh, self.integrals, self.vel = self.disc.mesh, self.disc.integrals, self.disc.vel
        self.bcdata = self.disc.bcdata
        self.ndir, self.n_tris, self.ndof = self.disc.ndir, self.disc.n_tris, self.disc.ndof
        self.precision = case.performance.precision
        self.ctx = SweepContext(self.disc, device=device)
        f64 = dict(dtype=torch.float64, device=self.device)
        self.vdf = torch.zeros((self.ndir, self.n_tris, self.ndof), **f64).as_subclass(HostReadable)
        self.mom = Moments.zeros(self.ndof, self.n_tris, device=self.device)
        self.t_old = torch.zeros(self.n_tris, **f64)
        self._res = torch.zeros(2, **f64)
        self.restart_info = self._apply_restart()
        self.graph_block = int(graph_block)
        self.acc = None
        if case.scheme.accflag == 1:
            from .gsis import GSIS
            self.acc = GSIS(self)
        sync(self.device)
        self.setup_seconds = time.perf_counter() - t0

    # -- restart (pybte/driver.py:99-141) ------------------------------------
    def _restart_stem(self) -> str:
        c = self.case
        return (f"VDFP{c.dg.deg}T{self.n_tris:3d}NP{c.velmesh.npole:2d}NA{c.velmesh.nazim:2d}"
                .replace(" ", ""))

    def _apply_restart(self) -> dict:
        """Load the restart file into ``vdf`` when ``restart.enabled``.  A
        default-named file left in ``basedir`` while restart is off is an
        error unless ``restart.error_on_stale`` is False (the Fortran would
        read it silently)."""
        r = self.case.restart
        default = Path(self.case.basedir) / f"{self._restart_stem()}.out"
        if not r.enabled:
            if r.error_on_stale and default.exists():
                raise FileExistsError(
                    f"a restart file {default} is present but restart is disabled; delete it, or set "
                    "restart.enabled or restart.error_on_stale explicitly")
            return {"enabled": False, "path": None, "sha256": None}
        path = Path(r.path) if r.path else default
        if not path.is_absolute():
            path = Path(self.case.basedir) / path
        if not path.exists():
            raise FileNotFoundError(f"restart enabled but {path} does not exist")
        raw = path.read_bytes()
        want = self.vdf.numel() * 8
        if len(raw) != want:
            raise ValueError(f"{path}: {len(raw)} bytes, expected {want} (wrong DEG / mesh / angular resolution?)")
        # Fortran VDF(l, i, j1, j2) with l fastest is the C-order (ndir, n_tris,
        # ndof) array with direction d = j2 * npole + j1: the same bytes.
        host = np.frombuffer(raw, dtype="<f8").astype(np.float64).reshape(tuple(self.vdf.shape))
        self.vdf.copy_(torch.from_numpy(host))
        return {"enabled": True, "path": str(path), "sha256": hashlib.sha256(raw).hexdigest()}

    def save_restart(self, path=None) -> Path:
        """Write ``vdf`` in the restart format; default name in ``basedir``."""
        path = Path(path) if path else Path(self.case.basedir) / f"{self._restart_stem()}.out"
        path.parent.mkdir(parents=True, exist_ok=True)
        path.write_bytes(self.vdf.detach().cpu().numpy().astype("<f8").tobytes())
        return path

    def vdf_fortran(self) -> np.ndarray:
        """Host view ``VDF(NDOF, N_TRIS, NPOLE, NAZIM)`` of the distribution."""
        npole, nazim = self.case.velmesh.npole, self.case.velmesh.nazim
        v = self.vdf.detach().cpu().numpy()
        return np.transpose(v.reshape(nazim, npole, self.n_tris, self.ndof), (3, 2, 1, 0))

    # -- output (pybte/driver.py:256-291) ------------------------------------
    def write_outputs(self, rec: "RunRecord") -> dict:
        """Write what ``case.output`` asks for under its ``dir``: the run
        record JSON, a ``RunTime.txt`` line, and the fields on the sampling
        grid as ``field.npz`` and/or Tecplot ``field.dat``.  Returns
        ``{artefact: path}``."""
        from .output import append_runtime_log, locate_points, sample_fields, sampling_grid, write_tecplot

        c = self.case
        o = c.output
        out = c.output_path()
        out.mkdir(parents=True, exist_ok=True)
        written = {}
        if o.run_record:
            written["run_record"] = str(rec.to_json(out / "run_record.json"))
        if o.runtime_log:
            written["runtime_log"] = str(append_runtime_log(
                out / "RunTime.txt", rec.scheme, c.flow.tau_r, c.flow.tau_n, self.n_tris, c.velmesh.npole,
                c.velmesh.nazim, rec.iterations, rec.wall_clock))
        if o.field:
            px, py = sampling_grid(o.field_nx, o.field_ny)
            triid = locate_points(self.mesh, px, py, device=self.device)
            missing = int(np.count_nonzero(triid < 0))
            if missing:
                warnings.warn(f"{missing} sampling points fell outside the mesh")
            uq = self.acc.uq if self.acc is not None else None
            cx, cy, dw = self.vel.flat()
            pT, pqx, pqy, pxx, pxy, pyy = sample_fields(self.mesh, self.disc.basis, self.vdf, cx, cy, dw,
                                                        c.flow.cv, px, py, triid, uq=uq, ndof_tri=self.ndof)
            if o.npz:
                np.savez_compressed(out / "field.npz", px=px, py=py, triid=triid, T=pT, qx=pqx, qy=pqy,
                                    Nxx=pxx, Nxy=pxy, Nyy=pyy)
                written["field_npz"] = str(out / "field.npz")
            if o.tecplot:
                written["field_dat"] = str(write_tecplot(out / "field.dat", px, py, [pT, pqx, pqy, pxx, pxy, pyy],
                                                         ["T", "qx", "qy", "Nxx", "Nxy", "Nyy"]))
        return written

    def release(self) -> None:
        """Free the solver's device state now -- Krylov operators and their
        graphs, the acceleration, the context -- under the device lock, so
        nothing is destroyed while another thread captures a graph.  The
        solver is unusable afterwards."""
        with device_lock:
            self.__dict__.pop("_krylov_cache", None)
            self.acc = None
            ctx = self.__dict__.pop("ctx", None)
            del ctx
            empty_graveyard()

    def reset(self) -> None:
        """Back to the zero initial state of a fresh solve (on the current
        stream)."""
        self.vdf.zero_()
        for k in ("ts", "qxs", "qys", "temp", "qx", "qy"):
            getattr(self.mom, k).zero_()
        self.t_old.zero_()
        self.ctx.flux_wall.zero_()

    # -- one outer iteration (pybte/driver.py:149-161) -----------------------
    def step(self, stream=None) -> None:
        if self.bcdata.has_nonthermalising:
            self.ctx.wall_flux(self.vdf, stream=stream)
        self.ctx.sweep(self.mom, self.vdf, stream=stream)
        if self.acc is None:
            self.ctx.moments(self.vdf, self.mom, stream=stream)
        else:
            self.acc.apply(stream=stream)

    def run(self, callback=None, progress_every: int = 0) -> RunRecord:
        rec = self._run(callback, progress_every)
        bad = self.ctx.singular_count(reset=True)
        if bad:
            # pybte's on-the-fly sweep would carry the inf/NaN on silently
            raise np.linalg.LinAlgError(f"{bad} zero pivots in the element operators during the run; "
                                        "check TAU_C and the mesh")
        return rec

    def _run(self, callback=None, progress_every: int = 0) -> RunRecord:
        """Solve to ``iteration.tol``.  ``callback(step, residual, solver)``
        after every outer step and ``progress_every`` progress lines, as
        pybte's (``driver.py:164-215``); either one, or
        ``iteration.true_residual``, moves CIS from the graph-captured loop
        to the host-driven one (same iterates, one host read per step)."""
        c = self.case
        if self.precision == "mixed":
            from .mixed import run_mixed
            return run_mixed(self)
        if c.scheme.method == "krylov":
            from .krylov import run_krylov
            return run_krylov(self, callback, progress_every)
        stepwise = callback is not None or progress_every or c.iteration.true_residual
        if self.acc is not None:
            device_loop = (getattr(self, "use_graphs", True) and c.performance.trace_solver == "device"
                           and not stepwise)
            if device_loop:
                return self._run_source("GSIS")
            return self._run_stepwise("GSIS", callback, progress_every)
        if stepwise:
            return self._run_stepwise("CIS", callback, progress_every)
        return self._run_source()

    # -- CIS and GSIS, graph-captured with a device stop flag ---------------
    def _iteration(self, s: int, tol: float, tmax: int, done, count, hist, cap) -> None:
        L = _lib.lib()
        ctx = self.ctx.handle
        if self.bcdata.has_nonthermalising:
            _lib.check(L.pbte_wall_flux(ctx, self.vdf.data_ptr(), self.ctx.flux_wall.data_ptr(), s), "wall_flux")
        m = self.mom
        _lib.check(L.pbte_sweep(ctx, m.ts.data_ptr(), m.qxs.data_ptr(), m.qys.data_ptr(), self.vdf.data_ptr(),
                                self.ctx.flux_wall.data_ptr(), self.ctx.pbuf.data_ptr(), 0, s), "sweep")
        if self.acc is None:
            _lib.check(L.pbte_moments(ctx, self.vdf.data_ptr(), m.ts.data_ptr(), m.qxs.data_ptr(),
                                      m.qys.data_ptr(), m.temp.data_ptr(), m.qx.data_ptr(), m.qy.data_ptr(), s),
                       "moments")
        else:
            self.acc.apply()   # on the current (capturing) stream, whose handle is s
        _lib.check(L.pbte_residual_iterate(ctx, m.temp.data_ptr(), self.t_old.data_ptr(),
                                           self._res.data_ptr(), s), "residual")
        _lib.check(L.pbte_residual_check(ctx, self._res.data_ptr(), float(tol), int(tmax), done.data_ptr(),
                                         count.data_ptr(), hist.data_ptr(), int(cap), s), "check")

    def _run_source(self, scheme: str = "CIS") -> RunRecord:
        """Blocks of ``graph_block`` iterations (CIS: sweep + moments; GSIS:
        sweep + the acceleration step) captured as one CUDA graph and replayed
        until the device stopping rule (pybte's step residual, ``driver.py:
        187-199``) sets the stop flag: every launch after it returns at once,
        so the state is the one of the converged iteration.  The host reads
        the flag once per block."""
        c = self.case
        tol, tmax = c.iteration.tol, c.iteration.tmax
        dev = self.device
        done = torch.zeros(1, dtype=torch.int32, device=dev)
        count = torch.zeros(1, dtype=torch.int64, device=dev)
        cap = min(int(tmax), 1 << 22)
        hist = torch.zeros(2 * cap, dtype=torch.float64, device=dev)
        L = _lib.lib()
        _lib.check(L.pbte_set_done_flag(self.ctx.handle, done.data_ptr()), "set_done_flag")
        if self.acc is not None:
            self.acc.done = done
        K = max(1, min(self.graph_block if self.acc is None else max(1, self.graph_block // 2), int(tmax)))
        stream = torch.cuda.Stream(device=dev)
        sync(dev)
        t0 = time.perf_counter()
        g = None
        try:
            g = torch.cuda.CUDAGraph()
            with device_lock:
                empty_graveyard()
                with torch.cuda.graph(g, stream=stream, capture_error_mode="thread_local"):
                    s = torch.cuda.current_stream().cuda_stream
                    for _ in range(K):
                        self._iteration(s, tol, tmax, done, count, hist, cap)
            while True:
                g.replay()
                if int(done.item()) != 0:
                    break
        finally:
            _lib.check(L.pbte_set_done_flag(self.ctx.handle, None), "set_done_flag")
            if self.acc is not None:
                self.acc.done = None
            bury(g)
        sync(dev)
        wall = time.perf_counter() - t0
        n = int(count.item())
        flag = int(done.item())
        self.ctx.sweep_count += n
        if self.acc is not None:
            # counted once per captured step at capture time, where nothing ran
            self.acc.solve_count += n - K
        h = hist[:2 * min(n, cap)].cpu().numpy().reshape(-1, 2)
        return self._record(n, flag == 1, h[:, 0], h[:, 1], wall, scheme)

    # -- host-driven loop (GSIS and debugging) -------------------------------
    def _run_stepwise(self, scheme: str, callback=None, progress_every: int = 0) -> RunRecord:
        c = self.case
        tol, tmax = c.iteration.tol, c.iteration.tmax
        want_true = c.iteration.true_residual
        every = max(1, int(c.iteration.true_residual_every))
        L = _lib.lib()
        residuals, masses, true_res = [], [], []
        sync(self.device)
        t0 = time.perf_counter()
        step, converged = 0, False
        s = torch.cuda.current_stream().cuda_stream

        def one_step(st):
            self.step(stream=st)
            _lib.check(L.pbte_residual_iterate(self.ctx.handle, self.mom.temp.data_ptr(), self.t_old.data_ptr(),
                                               self._res.data_ptr(), st.cuda_stream), "residual")

        # a GSIS step (dozens of launches: sweep, hot source, trace solve,
        # recovery, correction) is captured once and replayed; the host reads
        # the residual after each replay for pybte's stopping rule
        graph = None
        if (self.acc is not None and getattr(self, "use_graphs", True)
                and c.performance.trace_solver == "device"):
            graph = torch.cuda.CUDAGraph()
            with device_lock:
                empty_graveyard()
                sync(self.device)
                with torch.cuda.graph(graph, stream=torch.cuda.Stream(device=self.device),
                                      capture_error_mode="thread_local"):
                    one_step(torch.cuda.current_stream())
            # counted at capture, where nothing ran
            self.acc.solve_count -= 1
            self.ctx.sweep_count -= 1
        while True:
            step += 1
            if graph is not None:
                graph.replay()
                self.acc.solve_count += 1
                self.ctx.sweep_count += 1
            else:
                one_step(torch.cuda.current_stream())
            r = self._res.cpu().numpy()
            res = float(r[0])
            residuals.append(res)
            masses.append(float(r[1]))
            if want_true:
                true_res.append(self.true_residual() if step % every == 0 else np.nan)
            if progress_every and step % progress_every == 0:
                print(f"  step {step:8d}  residual {res:.6e}  mass {masses[-1]:.10f}", flush=True)
            if callback is not None:
                callback(step, res, self)
            if res < tol:
                converged = True
                break
            if step >= tmax:
                break
        sync(self.device)
        bury(graph)
        wall = time.perf_counter() - t0
        return self._record(step, converged, np.array(residuals), np.array(masses), wall, scheme,
                            true_res=true_res if want_true else None)

    def _record(self, iterations, converged, residuals, masses, wall, scheme, extra=None,
                true_res=None) -> RunRecord:
        c = self.case
        h = self.mom.host()
        nfact = self.ndir * self.n_tris
        if self.ctx.mode != "precomputed":
            # pybte counts on-the-fly factorisations in its Krylov products only
            nfact = nfact * self.ctx.sweep_count if scheme == "KRYLOV" else 0
        rec = RunRecord(iterations=int(iterations), converged=bool(converged),
                        residual_history=np.asarray(residuals),
                        residual_true=np.asarray(true_res) if true_res is not None else None,
                        mass_history=np.asarray(masses),
                        temp=h["temp"], qx=h["qx"], qy=h["qy"], temp_dofs=h["ts"], qx_dofs=h["qxs"],
                        qy_dofs=h["qys"], sweep_count=self.ctx.sweep_count, factorisation_count=int(nfact),
                        wall_clock=wall, setup_wall_clock=self.setup_seconds, config_hash=c.config_hash,
                        scheme=scheme, acc_variant=c.scheme.acc_variant if c.scheme.accflag == 1 else None,
                        tol=c.iteration.tol, tmax=c.iteration.tmax, tau_r=c.flow.tau_r, tau_n=c.flow.tau_n,
                        tau_c=c.tau_c, deg=c.dg.deg, npole=c.velmesh.npole, nazim=c.velmesh.nazim,
                        n_tris=self.n_tris, n_faces=self.mesh.n_faces, mesh_file=str(c.mesh_path()),
                        restart=dict(self.restart_info), environment=RunRecord.environment_fingerprint(),
                        precision=self.precision,
                        diagnostics={"sweep_mode": self.ctx.mode, "cycles_broken": 0,
                                     "hmin": float(self.mesh.hmin), "n_faces_b": int(self.mesh.n_faces_b),
                                     "boundary_types": [b.type for b in c.boundaries],
                                     "n_classes": self.ctx.n_classes, "n_levels_max": self.ctx.n_levels_max,
                                     "device_bytes": self.ctx.device_bytes})
        if self.acc is not None and hasattr(self.acc, "diagnostics"):
            rec.diagnostics.update(self.acc.diagnostics())
        if extra:
            rec.diagnostics.update(extra)
        return rec

    def true_residual(self) -> float:
        return self.ctx.true_residual(self.mom, self.vdf)
