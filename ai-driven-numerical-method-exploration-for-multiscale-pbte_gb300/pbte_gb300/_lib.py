"""ctypes binding of ``libpbte_gb300.so`` (the C ABI declared in
``include/pbte_gb300.h``) and its in-tree build.

The library is the only compute path: if it is missing or fails to load,
every GPU entry point raises -- there is no CPU fallback.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
from pathlib import Path

PKG_ROOT = Path(__file__).resolve().parent.parent          # holds csrc/ and _build/
REPO_ROOT = PKG_ROOT.parent
CSRC = PKG_ROOT / "csrc"
INCLUDE = REPO_ROOT / "include"
LIB_PATH = PKG_ROOT / "_build" / "libpbte_gb300.so"
SOURCES = ["pbte_ctx.cu", "pbte_kernels.cu", "pbte_sweep.cu", "pbte_krylov.cu", "pbte_capi.cu",
           "pbte_noalloc.cu", "pbte_output.cu", "pbte_trace.cu", "pbte_gsis.cu"]
ARCH = "-gencode=arch=compute_103a,code=sm_103a"

PBTE_OK = 0
MAX_BASIS = 1024           # PBTE_MAX_BASIS


def cgs2_scratch(rows: int) -> int:
    """PBTE_CGS2_SCRATCH_ROWS(rows): doubles of scratch a CGS2 over ``rows``
    basis rows needs."""
    return 8 + 2 * MAX_BASIS + 1216 * ((rows + 7) // 8 * 8)


CGS2_SCRATCH = cgs2_scratch(64)   # PBTE_CGS2_SCRATCH
ERRORS = {-1: "bad argument", -2: "CUDA runtime error", -3: "sweep graph has a cycle",
          -4: "configuration not supported", -5: "device wait timed out",
          -6: "singular element operator", -7: "device allocation failed"}


class PbteError(RuntimeError):
    def __init__(self, code: int, what: str):
        self.code = code
        super().__init__(f"{what}: {ERRORS.get(code, 'error')} (status {code})")


def _sources() -> list[Path]:
    return [CSRC / s for s in SOURCES if (CSRC / s).exists()]


def build(force: bool = False, verbose: bool = False) -> Path:
    """Compile the library for sm_103a with nvcc (one shared object)."""
    srcs = _sources()
    deps = srcs + list(CSRC.glob("*.cuh")) + [INCLUDE / "pbte_gb300.h"]
    if LIB_PATH.exists() and not force:
        t = LIB_PATH.stat().st_mtime
        if all(p.stat().st_mtime <= t for p in deps):
            return LIB_PATH
    LIB_PATH.parent.mkdir(exist_ok=True)
    nvcc = os.environ.get("NVCC", "nvcc")
    objs = []
    procs = []
    for s in srcs:
        o = LIB_PATH.parent / (s.stem + ".o")
        objs.append(o)
        # host code without FMA contraction: the schedule's inflow signs and
        # pybte's element order are computed as numpy computes them
        cmd = [nvcc, ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-ffp-contract=off", "-c",
               f"-I{INCLUDE}", f"-I{CSRC}", str(s), "-o", str(o)]
        procs.append((cmd, subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)))
    for cmd, p in procs:
        out, _ = p.communicate()
        if p.returncode != 0:
            raise RuntimeError(f"nvcc failed: {' '.join(cmd)}\n{out.decode()}")
        if verbose:
            print(out.decode())
    tmp = LIB_PATH.with_suffix(f".{os.getpid()}.tmp")
    subprocess.run([nvcc, ARCH, "-shared", "-o", str(tmp)] + [str(o) for o in objs]
                   + ["-lcudart"], check=True)
    os.replace(tmp, LIB_PATH)
    return LIB_PATH


_d = ctypes.POINTER(ctypes.c_double)
_i32 = ctypes.POINTER(ctypes.c_int32)
_vp = ctypes.c_void_p


class CaseDesc(ctypes.Structure):
    """Mirror of ``pbte_case_desc``."""
    _fields_ = [("n_tris", ctypes.c_int32), ("n_faces", ctypes.c_int32), ("ndof", ctypes.c_int32),
                ("ndof_fc", ctypes.c_int32), ("ndir", ctypes.c_int32), ("nbc", ctypes.c_int32),
                ("cv", ctypes.c_double), ("vg", ctypes.c_double), ("tau_r", ctypes.c_double),
                ("tau_n", ctypes.c_double), ("tau_c", ctypes.c_double),
                ("cxv", _d), ("cyv", _d), ("domega", _d),
                ("ref_mass", _d), ("ref_dx", _d), ("ref_dy", _d), ("ref_edge", _d),
                ("edge_dofs", _i32), ("area2", _d), ("dxi", _d), ("deta", _d),
                ("edge_scale", _d), ("nx", _d), ("ny", _d), ("tri_faces", _i32),
                ("upwind_tri", _i32), ("edge_map", _i32), ("face_bc", _i32),
                ("face_tri", _i32), ("face_lfc", _i32), ("bc_type", _i32), ("bc_temp", _d),
                ("int_tri", _d)]


class GmresCycleF32(ctypes.Structure):
    """Mirror of ``pbte_gmres_cycle_f32`` (the buffers of
    ``pbte_gmres_columns_f32``)."""
    _fields_ = [("ts", _vp), ("qxs", _vp), ("qys", _vp), ("flux_wall_in", _vp),
                ("wall_scale", ctypes.c_double), ("vdf32", _vp),
                ("ts_out", _vp), ("qxs_out", _vp), ("qys_out", _vp), ("flux_wall_out", _vp),
                ("temp", _vp), ("qx", _vp), ("qy", _vp),
                ("Q", _vp), ("ldq", ctypes.c_int64), ("uout", _vp), ("g", _vp), ("uin", _vp), ("w", _vp),
                ("n", ctypes.c_int64), ("h", _vp), ("scratch", _vp), ("scratch_len", ctypes.c_int64),
                ("R", _vp), ("ldr", ctypes.c_int32), ("cs", _vp), ("sn", _vp), ("gam", _vp),
                ("tol_abs", _vp), ("state", _vp), ("hist", _vp)]


class GsisOps(ctypes.Structure):
    """Mirror of ``pbte_gsis_ops`` (the field-major static-condensation
    operators of the GSIS step)."""
    _fields_ = [("n_tris", ctypes.c_int32), ("n_faces", ctypes.c_int32), ("ndof", ctypes.c_int32),
                ("ndof_fc", ctypes.c_int32), ("variant", ctypes.c_int32), ("n2", ctypes.c_int32),
                ("n_walls", ctypes.c_int32), ("pad", ctypes.c_int32), ("cv", ctypes.c_double),
                ("inv_t", _vp), ("ba1_t", _vp), ("tri1", _vp), ("ba2_t", _vp), ("slot2", _vp), ("tri2", _vp),
                ("mirror2", _vp), ("wall_slot", _vp), ("wall_kind", _vp), ("wall_nx", _vp), ("wall_ny", _vp),
                ("aa_trace_t", _vp), ("tri_faces", _vp)]


class BatchItem(ctypes.Structure):
    """Mirror of ``pbte_batch_item``."""
    _fields_ = [("ctx", _vp), ("ts", _vp), ("qxs", _vp), ("qys", _vp), ("flux_wall", _vp),
                ("wall_scale", ctypes.c_double), ("vdf32", _vp), ("done", _vp)]


_SIGS = {
    "pbte_ctx_create": ([ctypes.POINTER(CaseDesc), ctypes.c_int, ctypes.POINTER(_vp)], ctypes.c_int),
    "pbte_ctx_destroy": ([_vp], ctypes.c_int),
    "pbte_direction_classes": ([ctypes.POINTER(CaseDesc), _vp, ctypes.POINTER(ctypes.c_int32)], ctypes.c_int),
    "pbte_direction_levels": ([ctypes.POINTER(CaseDesc), ctypes.c_int32, _vp, ctypes.POINTER(ctypes.c_int32)],
                              ctypes.c_int),
    "pbte_ctx_info": ([_vp, ctypes.POINTER(ctypes.c_int64), ctypes.POINTER(ctypes.c_int64),
                       ctypes.POINTER(ctypes.c_int64)], ctypes.c_int),
    "pbte_sweep": ([_vp, _vp, _vp, _vp, _vp, _vp, _vp, ctypes.c_int, _vp], ctypes.c_int),
    "pbte_sweep_f32": ([_vp, _vp, _vp, _vp, _vp, _vp, ctypes.c_double, _vp], ctypes.c_int),
    "pbte_fixed_point_f32": ([_vp, _vp, _vp, _vp, _vp, ctypes.c_double] + [_vp] * 8 + [_vp], ctypes.c_int),
    "pbte_moments": ([_vp] + [_vp] * 7 + [_vp], ctypes.c_int),
    "pbte_moments_f32": ([_vp] + [_vp] * 7 + [_vp], ctypes.c_int),
    "pbte_wall_flux": ([_vp, _vp, _vp, _vp], ctypes.c_int),
    "pbte_wall_flux_f32": ([_vp, _vp, _vp, _vp], ctypes.c_int),
    "pbte_residual_iterate": ([_vp, _vp, _vp, _vp, _vp], ctypes.c_int),
    "pbte_set_done_flag": ([_vp, _vp], ctypes.c_int),
    "pbte_set_sweep_variant": ([_vp, ctypes.c_int], ctypes.c_int),
    "pbte_set_ring_groups": ([_vp, ctypes.c_int], ctypes.c_int),
    "pbte_set_ring_width": ([_vp, ctypes.c_int], ctypes.c_int),
    "pbte_ctx_schedule": ([_vp, ctypes.POINTER(ctypes.c_int64), ctypes.POINTER(ctypes.c_int64),
                           ctypes.POINTER(ctypes.c_int64)], ctypes.c_int),
    "pbte_residual_check": ([_vp, _vp, ctypes.c_double, ctypes.c_int64, _vp, _vp, _vp,
                             ctypes.c_int64, _vp], ctypes.c_int),
    "pbte_transport_residual": ([_vp] * 9 + [_vp], ctypes.c_int),
    "pbte_transport_residual_noalloc": ([_vp] * 8 + [_vp], ctypes.c_int),
    "pbte_cgs2": ([_vp, ctypes.c_int64, ctypes.c_int32, _vp, ctypes.c_int64, _vp, _vp, ctypes.c_int64, _vp],
                  ctypes.c_int),
    "pbte_cgs2_f32": ([_vp, ctypes.c_int64, ctypes.c_int32, _vp, ctypes.c_int64, _vp, _vp, ctypes.c_int64, _vp],
                      ctypes.c_int),
    "pbte_arnoldi_column": ([_vp, ctypes.c_int64, ctypes.c_int32, _vp, _vp, _vp, ctypes.c_int64, _vp, _vp,
                             ctypes.c_int64, _vp, _vp], ctypes.c_int),
    "pbte_arnoldi_column_f32": ([_vp, ctypes.c_int64, ctypes.c_int32, _vp, _vp, _vp, ctypes.c_int64, _vp, _vp,
                                 ctypes.c_int64, _vp, _vp], ctypes.c_int),
    "pbte_gmres_givens": ([ctypes.c_int32, _vp, _vp, ctypes.c_int32, _vp, _vp, _vp, _vp, _vp, _vp, _vp],
                          ctypes.c_int),
    "pbte_gmres_givens_bounded": ([ctypes.c_int32, _vp, _vp, ctypes.c_int32, _vp, _vp, _vp, _vp, _vp, _vp, _vp],
                                  ctypes.c_int),
    "pbte_arnoldi_column_givens": ([_vp, ctypes.c_int64, ctypes.c_int32, _vp, _vp, _vp, ctypes.c_int64, _vp, _vp,
                                    ctypes.c_int64, _vp, ctypes.c_int32, _vp, _vp, _vp, _vp, _vp, _vp,
                                    ctypes.c_int32, _vp], ctypes.c_int),
    "pbte_gmres_next_basis": ([ctypes.c_int32, _vp, _vp, _vp, ctypes.c_int64, _vp, ctypes.c_int64, _vp, _vp],
                              ctypes.c_int),
    "pbte_gmres_next_basis_f32": ([ctypes.c_int32, _vp, _vp, _vp, ctypes.c_int64, _vp, ctypes.c_int64, _vp, _vp],
                                  ctypes.c_int),
    "pbte_gmres_columns_f32": ([_vp, ctypes.POINTER(GmresCycleF32), ctypes.c_int32, ctypes.c_int32, _vp],
                               ctypes.c_int),
    "pbte_hot_source": ([_vp, _vp, ctypes.c_double, _vp, _vp], ctypes.c_int),
    "pbte_wall_trace": ([_vp, _vp, _vp, ctypes.c_int32, _vp, _vp, _vp, _vp], ctypes.c_int),
    "pbte_correct": ([_vp, _vp, _vp, _vp, ctypes.c_double, ctypes.c_int] + [_vp] * 6 + [_vp],
                     ctypes.c_int),
    "pbte_batched_inverse": ([_vp, _vp, ctypes.c_int32, ctypes.c_int32, _vp, _vp], ctypes.c_int),
    "pbte_nd_forward": ([_vp, ctypes.c_int32, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, ctypes.c_int32, _vp, _vp],
                        ctypes.c_int),
    "pbte_nd_backward": ([_vp, ctypes.c_int32, _vp, _vp, _vp, _vp, _vp, ctypes.c_int32, _vp, _vp], ctypes.c_int),
    "pbte_gsis_hot_apply": ([_vp, ctypes.POINTER(GsisOps), _vp, ctypes.c_double, _vp, _vp], ctypes.c_int),
    "pbte_gsis_apply_inverse": ([ctypes.POINTER(GsisOps), _vp, ctypes.c_int32, ctypes.c_int32, _vp, _vp, _vp],
                                ctypes.c_int),
    "pbte_gsis_trace_rhs": ([ctypes.POINTER(GsisOps), _vp, _vp, _vp, _vp, _vp], ctypes.c_int),
    "pbte_gsis_local_recover": ([ctypes.POINTER(GsisOps), _vp, _vp, _vp, _vp, _vp], ctypes.c_int),
    "pbte_sweep_fold_f32": ([_vp, _vp, _vp, _vp, _vp, ctypes.c_double, _vp, _vp], ctypes.c_int),
    "pbte_fold_epilogue_f32": ([_vp] * 9 + [_vp], ctypes.c_int),
    "pbte_gsis_hot_apply_f32": ([_vp, ctypes.POINTER(GsisOps), _vp, ctypes.c_double, _vp, _vp], ctypes.c_int),
    "pbte_wall_trace_f32": ([_vp, _vp, _vp, ctypes.c_int32, _vp, _vp, _vp, _vp], ctypes.c_int),
    "pbte_correct_f32": ([_vp, _vp, _vp, _vp, ctypes.c_double, ctypes.c_int, _vp, _vp, _vp, _vp], ctypes.c_int),
    "pbte_sweep_batch_create": ([ctypes.c_int32, ctypes.POINTER(BatchItem), ctypes.c_int32, ctypes.c_int32,
                                 ctypes.POINTER(_vp)], ctypes.c_int),
    "pbte_sweep_batch_run": ([_vp, ctypes.c_int, _vp], ctypes.c_int),
    "pbte_sweep_batch_destroy": ([_vp], ctypes.c_int),
    "pbte_singular_count": ([_vp, ctypes.POINTER(ctypes.c_int64), ctypes.c_int], ctypes.c_int),
    "pbte_device_bytes_live": ([ctypes.POINTER(ctypes.c_int64)], ctypes.c_int),
    "pbte_factorise_f32": ([_vp, _vp], ctypes.c_int),
    "pbte_periodic_count": ([_vp, ctypes.POINTER(ctypes.c_int64)], ctypes.c_int),
    "pbte_periodic_gather": ([_vp, _vp, _vp, _vp], ctypes.c_int),
    "pbte_periodic_scatter": ([_vp, _vp, _vp, _vp], ctypes.c_int),
    "pbte_field_moments": ([_vp, ctypes.c_int32, ctypes.c_int32, ctypes.c_int32] + [_vp] * 6 + [_vp],
                           ctypes.c_int),
    "pbte_locate_points": ([_vp, _vp, ctypes.c_int32, ctypes.c_double, ctypes.c_double, ctypes.c_double,
                            ctypes.c_double, ctypes.c_int32, ctypes.c_int32, _vp, _vp, _vp, ctypes.c_int32,
                            _vp, ctypes.c_int32, _vp, _vp], ctypes.c_int),
    "pbte_sample_fields": ([_vp, _vp, _vp, _vp, ctypes.c_int32, _vp, ctypes.c_int32, _vp, _vp, ctypes.c_int32,
                            _vp, _vp, _vp, ctypes.c_int32, ctypes.c_double, _vp, _vp, _vp], ctypes.c_int),
    "pbte_version": ([], ctypes.c_char_p),
}

_lib = None


def lib():
    """Load (building first if needed) the library; raises if unavailable."""
    global _lib
    if _lib is not None:
        return _lib
    if not LIB_PATH.exists():
        build()
    try:
        handle = ctypes.CDLL(str(LIB_PATH))
    except OSError as e:
        raise RuntimeError(f"cannot load {LIB_PATH}: {e}; the GPU path has no fallback") from e
    for name, (args, res) in _SIGS.items():
        fn = getattr(handle, name, None)
        if fn is None:
            continue
        fn.argtypes = args
        fn.restype = res
    _lib = handle
    return _lib


def check(status: int, what: str) -> None:
    if status != PBTE_OK:
        raise PbteError(status, what)


def exported_symbols() -> list[str]:
    return [n for n in _SIGS]
