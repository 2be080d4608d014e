"""Case validation against pybte's: every case dictionary of the fixture
(tests/golden/config_errors.json, written by make_golden.py --config-only
from pybte's own Case.from_dict) loads or fails here as it does in pybte,
with the same exception type, and the loaded ones carry the same coerced
values (tol from a string, nazim made even, the kernel name lower-cased)."""
import json
from pathlib import Path

import pytest

from pbte_gb300.config import Case

FIXTURE = Path(__file__).resolve().parent / "golden" / "config_errors.json"
ENTRIES = json.loads(FIXTURE.read_text())


@pytest.mark.parametrize("entry", ENTRIES, ids=[e["label"] for e in ENTRIES])
def test_case_validation_matches_pybte(entry):
    try:
        c = Case.from_dict(entry["case"])
        codes = [b.code for b in c.boundaries]
        result = "ok"
    except Exception as e:       # the exception type is what is compared
        result = type(e).__name__
    assert result == entry["result"]
    if result == "ok":
        v = entry["values"]
        assert codes == entry["codes"]
        assert (c.iteration.tol, c.iteration.tmax, c.velmesh.nazim) == (v["tol"], v["tmax"], v["nazim"])
        if "performance" in entry["case"]:
            assert c.performance.kernel == v["kernel"]
