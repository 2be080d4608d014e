"""Fixtures of the 8192-triangle benchmark square, computed by the oracle.

The square of the solve benchmark: uniform 64 x 64 grid (8192 triangles), DG
P2, 256 ordinates (npole 8 x nazim 32), west/east isothermal at +0.5/-0.5,
north/south diffuse adiabatic, Kn_N = 0.1 Kn_R.  The oracle (``oracle/``, the
C/numpy restatement pinned to pybte by the other fixtures) runs here:

* GMRES(30) to 1e-8 at Kn_R = 10, 1, 0.1 (sweep counts and fields: the FP64
  GPU solve must match them within one sweep and 1e-10 relative L2);
* GMRES without restart (basis up to 1023) to 1e-12 at the same Kn_R: the
  fixed point the mixed-precision solve is measured against;
* CIS to 1e-8 at Kn_R = 10, GSIS to 1e-8 at Kn_R = 0.01.

Element fields only (temperature deviation, heat flux), about 1 MB.  Takes a
few minutes on an 8-core host:

    python tests/golden/make_c2_fixtures.py [--threads N]
"""
from __future__ import annotations

import json
import sys
import time
from pathlib import Path

import numpy as np

OUT = Path(__file__).resolve().parent
ROOT = OUT.parent.parent
sys.path[:0] = [str(ROOT), str(ROOT / "ai-driven-numerical-method-exploration-for-multiscale-pbte_gb300")]

from oracle.oracle import Oracle  # noqa: E402
from pbte_gb300.config import square_case  # noqa: E402
from pbte_gb300.discretisation import Discretisation  # noqa: E402

N, DEG, NPOLE, NAZIM = 64, 2, 8, 32


def main(threads: int) -> None:
    arrays, meta = {}, {}

    def keep(name, o, rec):
        arrays[f"{name}__temp"] = o.temp.copy()
        arrays[f"{name}__qx"] = o.qx.copy()
        arrays[f"{name}__qy"] = o.qy.copy()
        meta[name] = {"iterations": int(rec["iterations"]), "converged": bool(rec["converged"]),
                      "seconds": round(float(rec.get("wall", 0.0)), 1)}
        print(name, meta[name], flush=True)

    for kn in (10.0, 1.0, 0.1):
        for tag, tol, basis in (("gmres30", 1e-8, 30), ("tight", 1e-12, 1023)):
            case = square_case(N, DEG, NPOLE, NAZIM, tau_r=kn, method="krylov", tol=tol, tmax=20000,
                               krylov_restart=basis)
            o = Oracle(Discretisation.build(case), nthreads=threads)
            t0 = time.perf_counter()
            rec = o.run_krylov(max_basis=basis)
            rec.setdefault("wall", time.perf_counter() - t0)
            keep(f"{tag}_kn{kn:g}", o, rec)
    o = Oracle(Discretisation.build(square_case(N, DEG, NPOLE, NAZIM, tau_r=10.0, tol=1e-8)), nthreads=threads)
    keep("cis_kn10", o, o.run_source())
    o = Oracle(Discretisation.build(square_case(N, DEG, NPOLE, NAZIM, tau_r=0.01, accflag=1, tol=1e-8)),
               nthreads=threads)
    keep("gsis_kn0.01", o, o.run_source(gsis=True))
    np.savez_compressed(OUT / "c2_square64_oracle.npz", **arrays)
    (OUT / "c2_square64_oracle.json").write_text(json.dumps(meta, indent=1, sort_keys=True))


if __name__ == "__main__":
    n = int(sys.argv[sys.argv.index("--threads") + 1]) if "--threads" in sys.argv else 8
    main(n)
