"""The command line (pybte's ``python -m pybte run/info`` with JSON case
files, plus ``square`` for the benchmark square)."""
import json
import os
import subprocess
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
PKG = ROOT / "ai-driven-numerical-method-exploration-for-multiscale-pbte_gb300"

CASE = {"iteration": {"tol": 1e-8, "tmax": 2000}, "velmesh": {"npole": 4, "nazim": 8}, "dg": {"deg": 1},
        "flow": {"cv": 1.0, "vg": 1.0, "tau_r": 1.0, "tau_n": 0.1}, "mesh": {"file": "cavity:5"},
        "boundaries": [{"name": "SWall", "phyid": 11, "type": "thermalising", "temp": 0.0},
                       {"name": "NWall", "phyid": 12, "type": "thermalising", "temp": 1.0},
                       {"name": "EWall", "phyid": 13, "type": "thermalising", "temp": 0.0},
                       {"name": "WWall", "phyid": 14, "type": "thermalising", "temp": 0.0}]}


def _cli(*args, cwd):
    env = {**os.environ, "PYTHONPATH": os.pathsep.join([str(PKG), os.environ.get("PYTHONPATH", "")])}
    return subprocess.run([sys.executable, "-m", "pbte_gb300", *args], cwd=cwd, capture_output=True, text=True,
                          env=env, timeout=600)


def test_info(tmp_path):
    (tmp_path / "case.json").write_text(json.dumps(CASE))
    r = _cli("info", "case.json", cwd=tmp_path)
    assert r.returncode == 0, r.stderr
    assert "triangles     50" in r.stdout and "config hash" in r.stdout


@pytest.mark.gpu
def test_run_writes_outputs(cuda, tmp_path):
    (tmp_path / "case.json").write_text(json.dumps({**CASE, "output": {"dir": "out", "tecplot": True}}))
    r = _cli("run", "case.json", cwd=tmp_path)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "(converged)" in r.stdout
    for name in ("run_record.json", "RunTime.txt", "field.npz", "field.dat"):
        assert (tmp_path / "out" / name).exists(), name
    assert json.loads((tmp_path / "out" / "run_record.json").read_text())["converged"] is True
