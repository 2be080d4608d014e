"""The C-ABI library builds, loads without a GPU, and exports every entry
point include/pbte_gb300.h declares (no compute calls here)."""
import ctypes
import re
from pathlib import Path

import pytest

from pbte_gb300 import _lib

HEADER = Path(__file__).resolve().parents[1] / "include" / "pbte_gb300.h"


def declared():
    text = HEADER.read_text()
    return sorted(set(re.findall(r"^\s*(?:int|const char \*)\s*(pbte_\w+)\s*\(", text, re.M)))


def test_header_declares_the_interface():
    names = declared()
    for n in ("pbte_ctx_create", "pbte_sweep", "pbte_moments", "pbte_wall_flux", "pbte_residual_iterate",
              "pbte_transport_residual", "pbte_hot_source", "pbte_correct"):
        assert n in names


def test_library_exports_every_declared_symbol():
    try:
        path = _lib.build()
    except (OSError, RuntimeError, FileNotFoundError) as e:   # no nvcc in this environment
        if not _lib.LIB_PATH.exists():
            pytest.skip(f"library not built and cannot build here: {e}")
        path = _lib.LIB_PATH
    handle = ctypes.CDLL(str(path))
    missing = [n for n in declared() if not hasattr(handle, n)]
    assert not missing, missing
    assert _lib.lib().pbte_version().decode().startswith("pbte_gb300")


def test_case_desc_matches_header_field_count():
    text = HEADER.read_text()
    body = text[text.index("typedef struct {"):text.index("} pbte_case_desc;")]
    decl = re.sub(r"/\*.*?\*/", "", body, flags=re.S)
    n = sum(len(re.findall(r"\*?\s*(\w+)\s*[,;]", line)) for line in decl.splitlines()
            if re.match(r"\s*(const\s+)?(int32_t|double)", line))
    assert n == len(_lib.CaseDesc._fields_)


def test_cgs2_rejects_short_scratch_on_the_host():
    """An undersized CGS2 scratch is refused before any launch (PBTE_ERR_ARG),
    so this runs without a GPU."""
    L = _lib.lib()
    buf = (ctypes.c_double * 16)()
    p = ctypes.cast(buf, ctypes.c_void_p)
    text = HEADER.read_text()
    assert f"#define PBTE_MAX_BASIS {_lib.MAX_BASIS}" in text
    assert "#define PBTE_CGS2_SCRATCH PBTE_CGS2_SCRATCH_ROWS(64)" in text
    assert "(8 + 2 * PBTE_MAX_BASIS + 1216 * ((((rows) + 7) / 8) * 8))" in text
    for rows in (1, 64, 200):
        short = _lib.cgs2_scratch(rows) - 1
        for fn in (L.pbte_cgs2, L.pbte_cgs2_f32):
            assert fn(p, 4, rows, p, 4, p, p, short, None) == -1
        for fn in (L.pbte_arnoldi_column, L.pbte_arnoldi_column_f32):
            assert fn(p, 4, rows, p, p, p, 4, p, p, short, None, None) == -1
    # a basis beyond PBTE_MAX_BASIS rows is refused whatever the scratch
    assert L.pbte_cgs2(p, 4, _lib.MAX_BASIS + 1, p, 4, p, p, 1 << 30, None) == -1


def test_gmres_cycle_struct_matches_header():
    """The ctypes mirror of pbte_gmres_cycle_f32 names the header's members
    in the header's order."""
    text = HEADER.read_text()
    end = text.index("} pbte_gmres_cycle_f32;")
    body = re.sub(r"/\*.*?\*/", "", text[text.rindex("typedef struct {", 0, end):end], flags=re.S)
    names = [m for line in body.splitlines()[1:] for m in re.findall(r"\**\s*(\w+)\s*(?=[,;])", line)]
    assert names == [f for f, _ in _lib.GmresCycleF32._fields_]


def test_gmres_columns_rejects_bad_arguments_on_the_host():
    L = _lib.lib()
    cyc = _lib.GmresCycleF32()
    assert L.pbte_gmres_columns_f32(None, ctypes.byref(cyc), 0, 1, None) == -1
    assert L.pbte_gmres_columns_f32(None, None, 0, 1, None) == -1
