"""Generate the golden fixtures under tests/golden/ from the reference itself.

Runs the reference solver (dingtao-shen/...-PBTE, ``solver-python/pybte``) in
its pure-Python/LAPACK mode (numba absent) and records its outputs on small
cases, plus the certified solutions shipped with the reference's benchmark
task (``tasks/t01-square/reference/*.npz``).  Needs the reference checkout,
so it runs only where that checkout exists.  Its location comes from the first
argument or from the environment variable ``PBTE_REFERENCE_ROOT``:

    PYTHONDONTWRITEBYTECODE=1 python tests/golden/make_golden.py <reference checkout>
    (sections alone: --config-only, --precond-only, --periodic-only, --field-only,
    --c1-only)

The fixtures are plain arrays; nothing at test time reads the reference.
"""
from __future__ import annotations

import atexit
import json
import os
import shutil
import sys
import tempfile
from pathlib import Path

import numpy as np

OUT = Path(__file__).resolve().parent


def _scratch() -> Path:
    """A temporary folder removed when the script exits."""
    d = tempfile.mkdtemp()
    atexit.register(shutil.rmtree, d, True)
    return Path(d)


def main(ref_root: str) -> None:
    ref = Path(ref_root)
    sys.path[:0] = [str(ref / "solver-python"), str(ref / "solver-python" / "tools")]
    from make_meshes import build
    from pybte import Case, Solver
    from pybte import krylov as rkrylov
    from pybte.acceleration import Acceleration  # noqa: F401  (import check)

    tmp = _scratch()
    mesh5 = tmp / "A1_Nx6_Ny6.msh"
    mesh5.write_text(build(5, "cavity", "smootherstep"))

    def case(deg, npole, nazim, tau_r, tau_n, south="nonthermalising", accflag=0,
             method="source", tol=1e-8, tmax=20000, north_t=1.0):
        return Case.from_dict({
            "iteration": {"tol": tol, "tmax": tmax},
            "scheme": {"accflag": accflag, "method": method},
            "velmesh": {"npole": npole, "nazim": nazim}, "dg": {"deg": deg},
            "flow": {"cv": 1.0, "vg": 1.0, "tau_r": tau_r, "tau_n": tau_n, "tau_thr": 1.0},
            "mesh": {"file": str(mesh5)},
            "boundaries": [{"name": "SWall", "phyid": 11, "type": south, "temp": 0.0},
                           {"name": "NWall", "phyid": 12, "type": "thermalising", "temp": north_t},
                           {"name": "EWall", "phyid": 13, "type": "thermalising", "temp": -0.5},
                           {"name": "WWall", "phyid": 14, "type": "thermalising", "temp": 0.5}],
            "output": {"field": False, "runtime_log": False, "run_record": False}}, basedir=str(tmp))

    meta = {}
    # 1. setup arrays + one sweep/moments/wall-flux/residual from seeded state
    for deg in (1, 2, 3):
        c = case(deg, 4, 8, 0.5, 0.05)
        s = Solver(c)
        ctx, it, m = s.ctx, s.integrals, s.mesh
        rng = np.random.default_rng(100 + deg)
        nd, nt = s.ndof, s.n_tris
        s.mom.ts[:] = rng.standard_normal((nd, nt))
        s.mom.qxs[:] = 0.3 * rng.standard_normal((nd, nt))
        s.mom.qys[:] = 0.3 * rng.standard_normal((nd, nt))
        vdf0 = rng.standard_normal(s.vdf.shape)
        s.vdf[:] = vdf0
        s.bcdata.update_wall_flux(s.vdf, ctx.cxv, ctx.cyv, ctx.domega, it.int_tri_fc, m)
        fw = s.bcdata.flux_wall.copy()
        ctx.sweep(s.mom, s.vdf)
        vdf1 = s.vdf.copy()
        tr = ctx.true_residual(s.mom, s.vdf)
        from pybte.moments import compute_moments
        compute_moments(s.vdf, ctx.cxv, ctx.cyv, ctx.domega, it.int_tri, 1.0, s.mom)
        np.savez_compressed(
            OUT / f"setup_sweep_deg{deg}.npz",
            nodes=m.nodes, tri_nodes=m.tri_nodes, tri_faces=m.tri_faces, face_nodes=m.face_nodes,
            face_bc=m.face_bc, face_tri=m.face_tri, face_lfc=m.face_lfc,
            tri_neighbour=m.tri_neighbour, tri_normal=m.tri_normal, tri_area=m.tri_area,
            face_len=m.face_len, tri_hmin=m.tri_hmin,
            int_tri=it.int_tri, int_tri_tri=it.int_tri_tri, int_tri_tri_x=it.int_tri_tri_x,
            int_tri_tri_y=it.int_tri_tri_y, int_tri_fc=it.int_tri_fc, int_tri_fc_fc=it.int_tri_fc_fc,
            int_fc_fc=it.int_fc_fc, int_fc=it.int_fc, int_tri_tri_fc=it.int_tri_tri_fc,
            cxv=ctx.cxv, cyv=ctx.cyv, domega=ctx.domega, order=ctx.order,
            ts_in=np.zeros(0), vdf_in=vdf0, flux_wall=fw, vdf_out=vdf1, true_residual=tr,
            ts_out=s.mom.ts, qxs_out=s.mom.qxs, qys_out=s.mom.qys, temp_out=s.mom.temp,
            qx_out=s.mom.qx, qy_out=s.mom.qy,
            ts_src=np.asarray(rng.bit_generator.state["state"]["state"] % 7))
        meta[f"setup_sweep_deg{deg}"] = {"deg": deg, "npole": 4, "nazim": 8, "tau_r": 0.5,
                                         "tau_n": 0.05, "seed": 100 + deg}
        print("setup/sweep deg", deg, "true residual", tr, flush=True)

    # 2. complete solves: CIS, GSIS, GMRES(30)
    runs = {
        "cis_deg1_adiabatic": dict(deg=1, npole=4, nazim=8, tau_r=1.0, tau_n=0.1),
        "cis_deg2_isothermal": dict(deg=2, npole=4, nazim=8, tau_r=0.3, tau_n=0.03,
                                    south="thermalising"),
        "gsis_deg2_adiabatic": dict(deg=2, npole=4, nazim=8, tau_r=0.1, tau_n=0.01, accflag=1),
        "gsis_deg1_isothermal": dict(deg=1, npole=4, nazim=8, tau_r=0.05, tau_n=0.005, accflag=1,
                                     south="thermalising"),
        "krylov_deg2_adiabatic": dict(deg=2, npole=4, nazim=8, tau_r=0.1, tau_n=0.01,
                                      method="krylov"),
    }
    orig_cap = rkrylov.krylov_basis_cap
    for name, kw in runs.items():
        if kw.get("method") == "krylov":
            rkrylov.krylov_basis_cap = lambda *a: 30
        c = case(**kw)
        s = Solver(c)
        rec = s.run()
        rkrylov.krylov_basis_cap = orig_cap
        np.savez_compressed(OUT / f"{name}.npz", iterations=rec.iterations,
                            converged=rec.converged, residuals=rec.residual_history,
                            masses=rec.mass_history, temp=rec.temp, qx=rec.qx, qy=rec.qy,
                            ts=rec.temp_dofs, qxs=rec.qx_dofs, qys=rec.qy_dofs,
                            true_residual=s.ctx.true_residual(s.mom, s.vdf))
        meta[name] = {**kw, "iterations": int(rec.iterations), "mass": float(rec.mass)}
        print(name, rec.iterations, rec.converged, rec.mass, flush=True)

    # 3. certified task solutions (GMRES to 1e-10 on the shipped 200-triangle mesh)
    task = ref / "tasks" / "t01-square"
    index = json.loads((task / "reference" / "index.json").read_text())
    keep = {}
    for key in ("F1_1_1", "F1_1e-1", "F2_1_1", "F2_1e-1"):
        z = np.load(task / "reference" / f"{key}.npz")
        keep[key] = {k: z[k] for k in ("temp", "qx", "qy", "temp_dofs")}
        meta[f"task_{key}"] = {"iterations": index[key]["iterations"],
                               "cis_iterations": index[key]["cis_iterations"],
                               "mass": index[key]["mass"]}
    np.savez_compressed(OUT / "task_solutions.npz",
                        **{f"{k}__{f}": v for k, d in keep.items() for f, v in d.items()})
    meta.update(field_output(ref, case))
    (OUT / "golden_meta.json").write_text(json.dumps(meta, indent=1, sort_keys=True))


def field_output(ref: Path, case) -> dict:
    """4. Field output, restart file and writers (``pybte/io_output.py``,
    ``pybte/driver.py:99-141``) on a converged GSIS solve, so the stress
    trio is non-zero; plus the shipped 200-triangle mesh's nodes and
    triangles, which the structured generator has to reproduce."""
    from pybte import Solver
    from pybte.io_output import (append_runtime_log, locate_points, sample_fields, sampling_grid,
                                 write_tecplot)
    from pybte.mesh.gmsh_reader import read_gmsh22

    tmp = _scratch()
    c = case(deg=2, npole=4, nazim=8, tau_r=0.1, tau_n=0.01, accflag=1)
    c.basedir = str(tmp)
    s = Solver(c)
    rec = s.run()
    px, py = sampling_grid()
    tri = locate_points(s.mesh, px, py)
    out = {"vdf": s.vdf, "uq": s.acc.uq, "px": px, "py": py, "triid": tri}
    for k, v in zip(("T", "qx", "qy", "Nxx", "Nxy", "Nyy"),
                    sample_fields(s.mesh, s.basis, s.vdf, s.ctx.cxv, s.ctx.cyv, s.ctx.domega,
                                  c.flow.cv, px, py, tri, uq=s.acc.uq, ndof_tri=s.ndof)):
        out[k] = v
    # a coarse grid that reaches outside the square, without the stress trio, cv = 2
    pxo, pyo = np.linspace(-0.05, 1.05, 23), np.linspace(-0.02, 1.02, 17)
    trio = locate_points(s.mesh, pxo, pyo)
    To, qxo, qyo, *_ = sample_fields(s.mesh, s.basis, s.vdf, s.ctx.cxv, s.ctx.cyv, s.ctx.domega,
                                     2.0, pxo, pyo, trio)
    out.update(pxo=pxo, pyo=pyo, triido=trio, To=To, qxo=qxo, qyo=qyo)
    # writers: Tecplot text of the coarse grid, RunTime.txt lines, restart bytes
    dat = write_tecplot(tmp / "field.dat", pxo, pyo, [To, qxo, qyo], ["T", "qx", "qy"])
    out["tecplot"] = np.frombuffer(dat.read_bytes(), dtype=np.uint8)
    log = tmp / "RunTime.txt"
    for args in (("CIS", 1e-3, 1e5, 200, 20, 40, 183211, 48123.46),
                 ("GSIS", 0.1, 0.01, 50, 4, 8, 17, 0.05),
                 ("KRYLOV", 2.5e-7, 3e12, 20000, 10, 20, 9, 123456789.0)):
        append_runtime_log(log, *args)
    out["runtime_log"] = np.frombuffer(log.read_bytes(), dtype=np.uint8)
    path = s.save_restart()
    out["restart"] = np.frombuffer(path.read_bytes(), dtype=np.uint8)
    # CIS restarted from that file (moments start at zero, the wall emission
    # from the loaded distribution)
    cr = case(deg=2, npole=4, nazim=8, tau_r=0.1, tau_n=0.01)
    cr.basedir = str(tmp)
    cr.restart.enabled = True
    cr.restart.path = str(path)
    sr = Solver(cr)
    # pybte leaves the loaded distribution as a read-only view of the file's
    # bytes, which its numpy sweep cannot write: run on a writable copy
    sr.vdf = sr.vdf.copy()
    rr = sr.run()
    out["restart_cis_temp"] = rr.temp
    out["restart_cis_residuals"] = rr.residual_history
    d = rec.to_dict(include_fields=False)
    out["record_keys"] = np.array(sorted(d))
    out["residuals"] = rec.residual_history
    shipped = read_gmsh22(ref / "solver-python" / "meshes" / "A1_Nx11_Ny11.msh")
    tri_ids = np.flatnonzero(shipped.elem_type == 2)
    line_ids = np.flatnonzero(shipped.elem_type == 1)
    out["shipped_nodes"] = shipped.nodes[:, :2]
    out["shipped_tri_nodes"] = np.array([shipped.elem_nodes[k] for k in tri_ids], dtype=np.int64)
    out["shipped_line_nodes"] = np.array([shipped.elem_nodes[k] for k in line_ids], dtype=np.int64)
    out["shipped_line_phyid"] = shipped.elem_phyid[line_ids]
    np.savez_compressed(OUT / "field_output.npz", **out)
    print("field output: restart", path.name, "iterations", rec.iterations, flush=True)
    return {"field_output": {"deg": 2, "npole": 4, "nazim": 8, "tau_r": 0.1, "tau_n": 0.01,
                             "accflag": 1, "iterations": int(rec.iterations),
                             "restart_name": path.name, "restart_cis_iterations": int(rr.iterations),
                             "contraction": rec.contraction, "error_estimate": rec.error_estimate,
                             "final_residual": rec.final_residual}}


def periodic(ref: Path) -> dict:
    """5. Periodic faces on the 5 x 5 channel (north T = 1, south T = 0,
    east/west a periodic pair): one seeded sweep in each of the reference's
    two periodic forms (partner read from the current vdf, or from pbuf),
    complete CIS / GSIS / GMRES(30) solves, the F3 task family's certified
    solutions, and the shipped channel mesh."""
    sys.path[:0] = [str(ref / "solver-python"), str(ref / "solver-python" / "tools")]
    from make_meshes import build
    from pybte import Case, Solver
    from pybte import krylov as rkrylov
    from pybte.mesh.gmsh_reader import read_gmsh22
    from pybte.moments import compute_moments

    tmp = _scratch()
    msh = tmp / "C1_Nx6_Ny6.msh"
    msh.write_text(build(5, "channel", "smootherstep", "uniform"))

    def case(deg, npole, nazim, tau_r, tau_n, accflag=0, method="source"):
        return Case.from_dict({
            "iteration": {"tol": 1e-8, "tmax": 20000}, "scheme": {"accflag": accflag, "method": method},
            "velmesh": {"npole": npole, "nazim": nazim}, "dg": {"deg": deg},
            "flow": {"cv": 1.0, "vg": 1.0, "tau_r": tau_r, "tau_n": tau_n, "tau_thr": 1.0},
            "mesh": {"file": str(msh)},
            "boundaries": [{"name": "SWall", "phyid": 11, "type": "thermalising", "temp": 0.0},
                           {"name": "NWall", "phyid": 12, "type": "thermalising", "temp": 1.0},
                           {"name": "Master", "phyid": 13, "type": "periodic", "temp": 0.0, "xoff": -1.0},
                           {"name": "Slave", "phyid": 14, "type": "periodic", "temp": 0.0, "xoff": 1.0}],
            "output": {"field": False, "runtime_log": False, "run_record": False}}, basedir=str(tmp))

    meta = {}
    out = {}
    for deg in (1, 2):
        s = Solver(case(deg, 4, 8, 0.5, 0.05))
        ctx = s.ctx
        rng = np.random.default_rng(200 + deg)
        nd, nt = s.ndof, s.n_tris
        s.mom.ts[:] = rng.standard_normal((nd, nt))
        s.mom.qxs[:] = 0.3 * rng.standard_normal((nd, nt))
        s.mom.qys[:] = 0.3 * rng.standard_normal((nd, nt))
        vdf0 = rng.standard_normal(s.vdf.shape)
        pbuf = rng.standard_normal(ctx.pbuf.shape)
        s.vdf[:] = vdf0
        ctx.sweep(s.mom, s.vdf)
        out[f"deg{deg}_vdf_in"] = vdf0
        out[f"deg{deg}_vdf_cis"] = s.vdf.copy()
        out[f"deg{deg}_true_residual"] = np.array(ctx.true_residual(s.mom, s.vdf))
        s.vdf[:] = vdf0
        ctx.pbuf[:] = pbuf
        ctx.use_pbuf = True
        ctx.sweep(s.mom, s.vdf)
        ctx.use_pbuf = False
        out[f"deg{deg}_pbuf"] = pbuf
        out[f"deg{deg}_vdf_pbuf"] = s.vdf.copy()
        out[f"deg{deg}_ts"], out[f"deg{deg}_qxs"], out[f"deg{deg}_qys"] = s.mom.ts, s.mom.qxs, s.mom.qys
        out[f"deg{deg}_periodic_tri"] = s.bcdata.periodic_tri
        meta[f"periodic_sweep_deg{deg}"] = {"deg": deg, "npole": 4, "nazim": 8, "tau_r": 0.5, "tau_n": 0.05,
                                            "seed": 200 + deg}
        print("periodic sweep deg", deg, flush=True)
    runs = {"cis_deg1": dict(deg=1, npole=4, nazim=8, tau_r=1.0, tau_n=0.1),
            "gsis_deg2": dict(deg=2, npole=4, nazim=8, tau_r=0.1, tau_n=0.01, accflag=1),
            "krylov_deg2": dict(deg=2, npole=4, nazim=8, tau_r=0.1, tau_n=0.01, method="krylov")}
    orig_cap = rkrylov.krylov_basis_cap
    for name, kw in runs.items():
        if kw.get("method") == "krylov":
            rkrylov.krylov_basis_cap = lambda *a: 30
        s = Solver(case(**kw))
        rec = s.run()
        rkrylov.krylov_basis_cap = orig_cap
        for k, v in (("temp", rec.temp), ("qx", rec.qx), ("qy", rec.qy), ("ts", rec.temp_dofs),
                     ("residuals", rec.residual_history)):
            out[f"{name}_{k}"] = v
        meta[f"periodic_{name}"] = {**kw, "iterations": int(rec.iterations), "mass": float(rec.mass),
                                    "converged": bool(rec.converged)}
        print("periodic", name, rec.iterations, rec.converged, rec.mass, flush=True)
    task = ref / "tasks" / "t01-square"
    index = json.loads((task / "reference" / "index.json").read_text())
    for key in ("F3_1_1", "F3_1e-1"):
        z = np.load(task / "reference" / f"{key}.npz")
        for f in ("temp", "qx", "qy", "temp_dofs"):
            out[f"task_{key}__{f}"] = z[f]
        meta[f"task_{key}"] = {"iterations": index[key]["iterations"],
                               "cis_iterations": index[key]["cis_iterations"], "mass": index[key]["mass"]}
    shipped = read_gmsh22(ref / "solver-python" / "meshes" / "C1_Nx11_Ny11.msh")
    tri_ids = np.flatnonzero(shipped.elem_type == 2)
    line_ids = np.flatnonzero(shipped.elem_type == 1)
    out["shipped_nodes"] = shipped.nodes[:, :2]
    out["shipped_tri_nodes"] = np.array([shipped.elem_nodes[k] for k in tri_ids], dtype=np.int64)
    out["shipped_line_nodes"] = np.array([shipped.elem_nodes[k] for k in line_ids], dtype=np.int64)
    out["shipped_line_phyid"] = shipped.elem_phyid[line_ids]
    np.savez_compressed(OUT / "periodic.npz", **out)
    _ = compute_moments
    return meta


def krylov_precond(ref: Path) -> dict:
    """6. GMRES(30) with pybte's moment preconditioner
    (``scheme.krylov_precond``, ``pybte/krylov.py:369-414``) on the 5 x 5
    cavity, diffusive (tau_R = 0.01) and ballistic (tau_R = 1) ends."""
    sys.path[:0] = [str(ref / "solver-python"), str(ref / "solver-python" / "tools")]
    from make_meshes import build
    from pybte import Case, Solver
    from pybte import krylov as rkrylov

    tmp = _scratch()
    msh = tmp / "A1_Nx6_Ny6.msh"
    msh.write_text(build(5, "cavity", "smootherstep"))
    meta, out = {}, {}
    orig_cap = rkrylov.krylov_basis_cap
    rkrylov.krylov_basis_cap = lambda *a: 30
    for name, tau_r in (("precond_diffusive", 0.01), ("precond_ballistic", 1.0)):
        c = Case.from_dict({
            "iteration": {"tol": 1e-8, "tmax": 20000},
            "scheme": {"accflag": 1, "method": "krylov", "krylov_precond": True},
            "velmesh": {"npole": 4, "nazim": 8}, "dg": {"deg": 1},
            "flow": {"cv": 1.0, "vg": 1.0, "tau_r": tau_r, "tau_n": 0.1 * tau_r, "tau_thr": 1.0},
            "mesh": {"file": str(msh)},
            "boundaries": [{"name": "SWall", "phyid": 11, "type": "thermalising", "temp": 0.0},
                           {"name": "NWall", "phyid": 12, "type": "thermalising", "temp": 1.0},
                           {"name": "EWall", "phyid": 13, "type": "thermalising", "temp": -0.5},
                           {"name": "WWall", "phyid": 14, "type": "thermalising", "temp": 0.5}],
            "output": {"field": False, "runtime_log": False, "run_record": False}}, basedir=str(tmp))
        rec = Solver(c).run()
        out[f"{name}_temp"] = rec.temp
        out[f"{name}_ts"] = rec.temp_dofs
        meta[name] = {"tau_r": tau_r, "iterations": int(rec.iterations), "converged": bool(rec.converged),
                      "mass": float(rec.mass)}
        print(name, rec.iterations, rec.converged, flush=True)
    rkrylov.krylov_basis_cap = orig_cap
    np.savez_compressed(OUT / "krylov_precond.npz", **out)
    return meta


def config_errors(ref: Path) -> None:
    """pybte's ``Case.from_dict`` on invalid and coerced case dictionaries:
    the exception type each raises (a boundary's type is checked when its
    code is read) and, where it loads, the coerced values; written to
    config_errors.json.  ``from_dict`` reads no mesh, so no file is needed."""
    sys.path[:0] = [str(ref / "solver-python")]
    import copy

    from pybte import Case

    walls = [{"name": "SWall", "phyid": 11, "type": "nonthermalising", "temp": 0.0},
             {"name": "NWall", "phyid": 12, "type": "thermalising", "temp": 1.0},
             {"name": "EWall", "phyid": 13, "type": "thermalising", "temp": -0.5},
             {"name": "WWall", "phyid": 14, "type": "thermalising", "temp": 0.5}]
    base = {"iteration": {"tol": 1e-8, "tmax": 100}, "scheme": {"accflag": 0},
            "velmesh": {"npole": 4, "nazim": 8}, "dg": {"deg": 2},
            "flow": {"cv": 1.0, "vg": 1.0, "tau_r": 1.0, "tau_n": 0.1, "tau_thr": 1.0},
            "mesh": {"file": "A1_Nx11_Ny11.msh"}, "boundaries": walls}
    variants = [
        ("valid", {}),
        ("tol as a string", {"iteration": {"tol": "1.0e-8", "tmax": "100"}}),
        ("odd nazim", {"velmesh": {"npole": 4, "nazim": 7}}),
        ("kernel upper case", {"performance": {"kernel": "NUMPY"}}),
        ("boundary type upper case", {"boundaries": [dict(walls[0], type="Thermalising")] + walls[1:]}),
        ("scheme.method", {"scheme": {"method": "multigrid"}}),
        ("scheme.krylov_max_bytes", {"scheme": {"krylov_max_bytes": 0}}),
        ("scheme.krylov_max_rounds", {"scheme": {"krylov_max_rounds": 0}}),
        ("scheme.defect_every", {"scheme": {"defect_every": -1}}),
        ("scheme.defect_anderson", {"scheme": {"defect_anderson": -2}}),
        ("scheme.defect_omega", {"scheme": {"defect_omega": 1.5}}),
        ("scheme.on_cycle", {"scheme": {"on_cycle": "ignore"}}),
        ("scheme.acc_variant", {"scheme": {"acc_variant": "C"}}),
        ("scheme.stabilisation", {"scheme": {"stabilisation": [1.0, 1.0]}}),
        ("flow.tau_r", {"flow": {"cv": 1.0, "vg": 1.0, "tau_r": 0.0, "tau_n": 0.1}}),
        ("flow.tau_n", {"flow": {"cv": 1.0, "vg": 1.0, "tau_r": 1.0, "tau_n": -0.1}}),
        ("flow.vg", {"flow": {"cv": 1.0, "vg": 0.0, "tau_r": 1.0, "tau_n": 0.1}}),
        ("velmesh.nazim", {"velmesh": {"npole": 4, "nazim": 1}}),
        ("dg.deg", {"dg": {"deg": 5}}),
        ("performance.kernel", {"performance": {"kernel": "opencl"}}),
        ("performance.threads", {"performance": {"threads": -1}}),
        ("boundary type", {"boundaries": [dict(walls[0], type="mirror")] + walls[1:]}),
        ("unknown key", {"flow": {"cv": 1.0, "vg": 1.0, "tau_r": 1.0, "tau_n": 0.1, "viscosity": 1.0}}),
        ("unknown boundary key", {"boundaries": [dict(walls[0], colour="red")] + walls[1:]}),
    ]
    out = []
    for label, mod in variants:
        d = copy.deepcopy(base)
        d.update(copy.deepcopy(mod))
        rec = {"label": label, "case": d}
        try:
            c = Case.from_dict(d)
            rec["codes"] = [b.code for b in c.boundaries]
            rec["result"] = "ok"
            rec["values"] = {"tol": c.iteration.tol, "tmax": c.iteration.tmax, "nazim": c.velmesh.nazim,
                             "kernel": c.performance.kernel}
        except Exception as e:                       # the type is the fixture
            rec["result"] = type(e).__name__
        out.append(rec)
    (OUT / "config_errors.json").write_text(json.dumps(out, indent=1, sort_keys=True))


def c1_square(ref: Path) -> dict:
    """The 800-triangle square of the CIS benchmark: uniform 20 x 20 grid, P1,
    64 ordinates (npole 4 x nazim 16), tau_R = 1, tau_N = 0.1, west/east
    isothermal at +0.5/-0.5, north/south diffuse adiabatic, CIS to 1e-8.
    About six minutes in pybte's pure-Python mode."""
    sys.path[:0] = [str(ref / "solver-python"), str(ref / "solver-python" / "tools")]
    from make_meshes import build
    from pybte import Case, Solver

    tmp = _scratch()
    (tmp / "U_20.msh").write_text(build(20, "cavity", "uniform"))
    c = Case.from_dict({
        "iteration": {"tol": 1e-8, "tmax": 5000}, "scheme": {"accflag": 0},
        "velmesh": {"npole": 4, "nazim": 16}, "dg": {"deg": 1},
        "flow": {"cv": 1.0, "vg": 1.0, "tau_r": 1.0, "tau_n": 0.1, "tau_thr": 1.0},
        "mesh": {"file": str(tmp / "U_20.msh")},
        "boundaries": [{"name": "SWall", "phyid": 11, "type": "nonthermalising", "temp": 0.0},
                       {"name": "NWall", "phyid": 12, "type": "nonthermalising", "temp": 0.0},
                       {"name": "EWall", "phyid": 13, "type": "thermalising", "temp": -0.5},
                       {"name": "WWall", "phyid": 14, "type": "thermalising", "temp": 0.5}],
        "output": {"field": False, "runtime_log": False, "run_record": False}}, basedir=str(tmp))
    s = Solver(c)
    rec = s.run()
    tr = s.ctx.true_residual(s.mom, s.vdf)
    np.savez_compressed(OUT / "c1_square20_cis.npz", iterations=rec.iterations, converged=rec.converged,
                        residuals=rec.residual_history, temp=rec.temp, qx=rec.qx, qy=rec.qy,
                        ts=rec.temp_dofs, qxs=rec.qx_dofs, qys=rec.qy_dofs, true_residual=tr)
    print("c1", rec.iterations, rec.converged, float(np.sum(rec.qx)), tr, flush=True)
    return {"c1_square20_cis": {"n": 20, "deg": 1, "npole": 4, "nazim": 16, "tau_r": 1.0, "tau_n": 0.1,
                                "iterations": int(rec.iterations), "true_residual": float(tr),
                                "sum_qx": float(np.sum(rec.qx))}}


if __name__ == "__main__":
    ref_root = sys.argv[1] if len(sys.argv) > 1 and not sys.argv[1].startswith("--") else \
        os.environ.get("PBTE_REFERENCE_ROOT")
    if not ref_root:
        sys.exit("usage: make_golden.py <reference checkout> [--section-only]  "
                 "(or set PBTE_REFERENCE_ROOT)")
    if "--c1-only" in sys.argv[1:]:
        m = json.loads((OUT / "golden_meta.json").read_text())
        m.update(c1_square(Path(ref_root)))
        (OUT / "golden_meta.json").write_text(json.dumps(m, indent=1, sort_keys=True))
    elif "--config-only" in sys.argv[1:]:
        config_errors(Path(ref_root))
    elif "--precond-only" in sys.argv[1:]:
        m = json.loads((OUT / "golden_meta.json").read_text())
        m.update(krylov_precond(Path(ref_root)))
        (OUT / "golden_meta.json").write_text(json.dumps(m, indent=1, sort_keys=True))
    elif "--periodic-only" in sys.argv[1:]:
        m = json.loads((OUT / "golden_meta.json").read_text())
        m.update(periodic(Path(ref_root)))
        (OUT / "golden_meta.json").write_text(json.dumps(m, indent=1, sort_keys=True))
    elif "--field-only" in sys.argv[1:]:
        sys.path[:0] = [str(Path(ref_root) / "solver-python"), str(Path(ref_root) / "solver-python" / "tools")]
        from make_meshes import build as _build
        from pybte import Case as _Case

        _tmp = _scratch()
        (_tmp / "A1_Nx6_Ny6.msh").write_text(_build(5, "cavity", "smootherstep"))

        def _case(deg, npole, nazim, tau_r, tau_n, accflag=0):
            return _Case.from_dict({
                "iteration": {"tol": 1e-8, "tmax": 20000}, "scheme": {"accflag": accflag},
                "velmesh": {"npole": npole, "nazim": nazim}, "dg": {"deg": deg},
                "flow": {"cv": 1.0, "vg": 1.0, "tau_r": tau_r, "tau_n": tau_n, "tau_thr": 1.0},
                "mesh": {"file": str(_tmp / "A1_Nx6_Ny6.msh")},
                "boundaries": [{"name": "SWall", "phyid": 11, "type": "nonthermalising", "temp": 0.0},
                               {"name": "NWall", "phyid": 12, "type": "thermalising", "temp": 1.0},
                               {"name": "EWall", "phyid": 13, "type": "thermalising", "temp": -0.5},
                               {"name": "WWall", "phyid": 14, "type": "thermalising", "temp": 0.5}],
                "output": {"field": False, "runtime_log": False, "run_record": False}}, basedir=str(_tmp))

        m = json.loads((OUT / "golden_meta.json").read_text())
        m.update(field_output(Path(ref_root), _case))
        (OUT / "golden_meta.json").write_text(json.dumps(m, indent=1, sort_keys=True))
    else:
        main(ref_root)
