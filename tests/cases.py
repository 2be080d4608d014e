"""Case builders shared by the tests (the fixtures' cases, restated)."""
from __future__ import annotations

import json
from pathlib import Path

import numpy as np

from pbte_gb300.config import Case

GOLDEN = Path(__file__).resolve().parent / "golden"


def golden(name: str):
    return np.load(GOLDEN / f"{name}.npz")


def meta() -> dict:
    return json.loads((GOLDEN / "golden_meta.json").read_text())


def small_case(deg, npole, nazim, tau_r, tau_n, south="nonthermalising", accflag=0, method="source",
               tol=1e-8, tmax=20000, north_t=1.0, mesh="cavity:5:smootherstep", precision="fp64",
               sweep_mode="auto", krylov_restart=None) -> Case:
    """The 50-triangle graded cavity of the fixtures: north wall at ``north_t``,
    east/west isothermal at -0.5/+0.5, south ``south``."""
    return Case.from_dict({
        "iteration": {"tol": tol, "tmax": tmax},
        "scheme": {"accflag": accflag, "method": method, "krylov_restart": krylov_restart},
        "velmesh": {"npole": npole, "nazim": nazim}, "dg": {"deg": deg},
        "flow": {"cv": 1.0, "vg": 1.0, "tau_r": tau_r, "tau_n": tau_n, "tau_thr": 1.0},
        "mesh": {"file": mesh},
        "boundaries": [{"name": "SWall", "phyid": 11, "type": south, "temp": 0.0},
                       {"name": "NWall", "phyid": 12, "type": "thermalising", "temp": north_t},
                       {"name": "EWall", "phyid": 13, "type": "thermalising", "temp": -0.5},
                       {"name": "WWall", "phyid": 14, "type": "thermalising", "temp": 0.5}],
        "performance": {"precision": precision, "sweep_mode": sweep_mode}})


def case_from_meta(name: str, **over) -> Case:
    m = dict(meta()[name])
    kw = {k: m[k] for k in ("deg", "npole", "nazim", "tau_r", "tau_n")}
    for k in ("south", "accflag", "method"):
        if k in m:
            kw[k] = m[k]
    kw.update(over)
    return small_case(**kw)


PERIODIC_EW = [{"name": "SWall", "phyid": 11, "type": "thermalising", "temp": 0.0},
               {"name": "NWall", "phyid": 12, "type": "thermalising", "temp": 1.0},
               {"name": "Master", "phyid": 13, "type": "periodic", "temp": 0.0, "xoff": -1.0},
               {"name": "Slave", "phyid": 14, "type": "periodic", "temp": 0.0, "xoff": 1.0}]


def periodic_case(deg, npole, nazim, tau_r, tau_n, accflag=0, method="source", tol=1e-8, tmax=20000,
                  mesh="channel:5:smootherstep", precision="fp64", sweep_mode="auto", krylov_restart=None) -> Case:
    """The periodic fixtures' channel: 50 triangles, uniform in x and graded
    in y, north T = 1, south T = 0, east/west a periodic pair."""
    return Case.from_dict({
        "iteration": {"tol": tol, "tmax": tmax},
        "scheme": {"accflag": accflag, "method": method, "krylov_restart": krylov_restart},
        "velmesh": {"npole": npole, "nazim": nazim}, "dg": {"deg": deg},
        "flow": {"cv": 1.0, "vg": 1.0, "tau_r": tau_r, "tau_n": tau_n, "tau_thr": 1.0},
        "mesh": {"file": mesh}, "boundaries": [dict(b) for b in PERIODIC_EW],
        "performance": {"precision": precision, "sweep_mode": sweep_mode}})


def task_case(family: str, tau: str, **over) -> Case:
    """The reference benchmark task's F1 / F2 / F3 cells: 200-triangle graded
    square, DEG 2, 10 x 20 ordinates, north wall T = 1, south T = 0; east /
    west isothermal at 0 (F1), diffuse adiabatic (F2), or a periodic pair on
    the channel mesh, uniform in x (F3)."""
    kn_r, kn_n = {"1_1": (1.0, 1.0), "1e-1": (0.1, 1e5)}[tau]
    ew = "thermalising" if family == "F1" else "nonthermalising"
    bnds = [{"name": "SWall", "phyid": 11, "type": "thermalising", "temp": 0.0},
            {"name": "NWall", "phyid": 12, "type": "thermalising", "temp": 1.0},
            {"name": "EWall", "phyid": 13, "type": ew, "temp": 0.0},
            {"name": "WWall", "phyid": 14, "type": ew, "temp": 0.0}]
    mesh = "cavity:10:smootherstep"
    if family == "F3":
        bnds, mesh = [dict(b) for b in PERIODIC_EW], "channel:10:smootherstep"
    d = {"iteration": {"tol": 1e-10, "tmax": 6000}, "scheme": {"method": "krylov"},
         "velmesh": {"npole": 10, "nazim": 20}, "dg": {"deg": 2},
         "flow": {"cv": 1.0, "vg": 1.0, "tau_r": kn_r, "tau_n": kn_n},
         "mesh": {"file": mesh}, "boundaries": bnds}
    for k, v in over.items():
        d.setdefault(k, {}).update(v) if isinstance(v, dict) else d.__setitem__(k, v)
    return Case.from_dict(d)
