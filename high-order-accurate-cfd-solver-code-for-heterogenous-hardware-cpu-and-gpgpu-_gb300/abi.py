"""ctypes binding of libcfd_gb300.so (include/cfd_rhs.h).

The product's compute path is the CUDA library; this module only declares
its C entry points.  Loading fails loudly when the library is missing: there
is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
import pathlib

from . import build as _build

LIB_PATH = _build.LIB

# status codes (cfd_status_t)
OK, EINVAL, ENONFINITE, ETIMEOUT, ECUDA, ENOMEM, EUNSUPPORTED = range(7)
STATUS_NAMES = {0: "CFD_OK", 1: "CFD_EINVAL", 2: "CFD_ENONFINITE", 3: "CFD_ETIMEOUT", 4: "CFD_ECUDA",
                5: "CFD_ENOMEM", 6: "CFD_EUNSUPPORTED"}
PATH_GATHER, PATH_STRUCTURED = 0, 1
PREC_FP64, PREC_MIXED, PREC_SPLIT = 0, 1, 2
PREC_NAMES = {PREC_FP64: "fp64", PREC_MIXED: "mixed", PREC_SPLIT: "split"}


class CfdError(RuntimeError):
    def __init__(self, status: int, where: str, detail: str = ""):
        self.status = status
        super().__init__(f"{where}: {STATUS_NAMES.get(status, status)}" + (f" ({detail})" if detail else ""))


class Params(C.Structure):
    _fields_ = [("mach", C.c_double), ("reynolds", C.c_double), ("prandtl", C.c_double), ("t_inf", C.c_double),
                ("weno_eps", C.c_double), ("viscous", C.c_int32), ("les", C.c_int32), ("precision", C.c_int32),
                ("reserved", C.c_int32), ("smagorinsky_cs", C.c_double)]


class Geometry(C.Structure):
    _fields_ = [("g_node", C.c_int32), ("sd_node", C.c_int32), ("grid", C.c_void_p), ("det", C.c_void_p),
                ("deter", C.c_void_p), ("metric", C.c_void_p)]


class KernelTime(C.Structure):
    _fields_ = [("name", C.c_char * 24), ("ms", C.c_double)]


class SolverInfo(C.Structure):
    _fields_ = [("path", C.c_int32), ("ni", C.c_int32), ("nj", C.c_int32), ("nk", C.c_int32),
                ("precision", C.c_int32), ("reserved", C.c_int32), ("device_bytes", C.c_uint64),
                ("face_tile_i", C.c_int32), ("face_tile_jk", C.c_int32), ("face_blocks", C.c_int32 * 3),
                ("reserved2", C.c_int32)]


class BatchInfo(C.Structure):
    _fields_ = [("n_active", C.c_int32), ("tile_nodes", C.c_int32), ("blocks", C.c_int32), ("graph", C.c_int32),
                ("precision", C.c_int32), ("n_held", C.c_int32), ("nodes_total", C.c_uint64),
                ("device_bytes", C.c_uint64), ("capacity_bytes", C.c_uint64), ("face_tiles", C.c_int32),
                ("reserved", C.c_int32)]


_vp = C.c_void_p
_i32 = C.c_int32
_d = C.c_double

# name -> (restype, argtypes)
PROTOTYPES = {
    "cfd_params_default": (None, [C.POINTER(Params)]),
    "cfd_status_string": (C.c_char_p, [C.c_int]),
    "cfd_last_error": (C.c_char_p, [_vp]),
    "cfd_ctx_create": (C.c_int, [C.POINTER(_vp), C.c_int]),
    "cfd_ctx_destroy": (C.c_int, [_vp]),
    "cfd_ctx_set_stream": (C.c_int, [_vp, _vp]),
    "cfd_ctx_set_async": (C.c_int, [_vp, C.c_int]),
    "cfd_ctx_synchronize": (C.c_int, [_vp]),
    "cfd_ctx_set_rows": (C.c_int, [_vp, _i32]),
    "cfd_ctx_set_face_reuse": (C.c_int, [_vp, C.c_int]),
    "cfd_ctx_launch_count": (C.c_uint64, [_vp]),
    "cfd_buffer_alloc": (C.c_int, [_vp, C.c_size_t, C.POINTER(_vp)]),
    "cfd_buffer_free": (C.c_int, [_vp, _vp]),
    "cfd_buffer_write": (C.c_int, [_vp, _vp, _vp, C.c_size_t]),
    "cfd_buffer_read": (C.c_int, [_vp, _vp, _vp, C.c_size_t]),
    "cfd_uq": (C.c_int, [_vp] + [_vp] * 6 + [_i32]),
    "cfd_viscous": (C.c_int, [_vp] + [_vp] * 11 + [_i32, C.POINTER(Params)]),
    "cfd_weno": (C.c_int, [_vp, _i32, _d, _d] + [_vp] * 16 + [_i32, C.POINTER(Params), _vp]),
    "cfd_solver_create": (C.c_int, [_vp, C.POINTER(Geometry), C.POINTER(Params), _i32, C.POINTER(_vp)]),
    "cfd_solver_destroy": (C.c_int, [_vp]),
    "cfd_solver_info": (C.c_int, [_vp, C.POINTER(SolverInfo)]),
    "cfd_solver_set_flow": (C.c_int, [_vp, _vp]),
    "cfd_solver_set_face_tiles": (C.c_int, [_vp, _i32, _i32]),
    "cfd_solver_set_face_blocks": (C.c_int, [_vp, _i32, _i32, _i32]),
    "cfd_solver_get_flow": (C.c_int, [_vp, _vp]),
    "cfd_solver_get_u0": (C.c_int, [_vp, _vp]),
    "cfd_solver_step": (C.c_int, [_vp, _d, _i32]),
    "cfd_solver_stage": (C.c_int, [_vp, _i32, _d, _vp]),
    "cfd_solver_profile_stage": (C.c_int, [_vp, _i32, _d, _vp, _i32, C.POINTER(_i32)]),
    "cfd_probe_flops": (C.c_int, [_vp, _i32, C.POINTER(_d)]),
    "cfd_probe_emu64": (C.c_int, [_vp, C.c_int64, C.c_uint64, C.POINTER(C.c_int64)]),
    "cfd_bc_create": (C.c_int, [_vp, _vp, _i32] + [_vp, _i32] * 4 + [C.POINTER(_vp)]),
    "cfd_bc_create_singular": (C.c_int, [_vp, _vp, _i32] + [_vp, _i32] * 4 + [_vp, _vp, _i32, C.POINTER(_vp)]),
    "cfd_bc_destroy": (C.c_int, [_vp]),
    "cfd_boundary_fill": (C.c_int, [_vp, _vp, _vp, _d, _i32, _i32]),
    "cfd_rk3_step": (C.c_int, [_vp, _d, _d] + [_vp] * 16 + [_i32, _i32, C.POINTER(Params), _vp, _i32]),
    "cfd_solver_set_boundary": (C.c_int, [_vp, _vp]),
    "cfd_batch_create": (C.c_int, [_vp, _i32, C.c_uint64, C.POINTER(_vp)]),
    "cfd_batch_destroy": (C.c_int, [_vp]),
    "cfd_batch_instance_bytes": (C.c_uint64, [_i32, C.c_int64]),
    "cfd_batch_add": (C.c_int, [_vp, C.POINTER(Geometry), C.POINTER(Params), _vp, _d, C.POINTER(_i32)]),
    "cfd_batch_remove": (C.c_int, [_vp, _i32]),
    "cfd_batch_stage": (C.c_int, [C.POINTER(Geometry), C.POINTER(Params), _vp, _d, C.POINTER(_vp)]),
    "cfd_batch_add_staged": (C.c_int, [_vp, _vp, C.POINTER(_i32)]),
    "cfd_batch_staged_free": (C.c_int, [_vp]),
    "cfd_batch_step": (C.c_int, [_vp, _i32]),
    "cfd_batch_step_async": (C.c_int, [_vp, _i32]),
    "cfd_batch_sync": (C.c_int, [_vp]),
    "cfd_batch_set_hold": (C.c_int, [_vp, _i32, _i32]),
    "cfd_batch_get_flow": (C.c_int, [_vp, _i32, _vp]),
    "cfd_batch_get_u0": (C.c_int, [_vp, _i32, _vp]),
    "cfd_batch_slot_status": (C.c_int, [_vp, _i32]),
    "cfd_batch_set_flow": (C.c_int, [_vp, _i32, _vp]),
    "cfd_batch_set_wait_limit": (C.c_int, [_vp, C.c_int64]),
    "cfd_batch_set_tiling": (C.c_int, [_vp, _i32, _i32, _i32]),
    "cfd_batch_tune": (C.c_int, [_vp, _i32]),
    "cfd_batch_info": (C.c_int, [_vp, C.POINTER(BatchInfo)]),
    "cfd_compact_metrics": (C.c_int, [_vp, _i32, _d, _vp, _vp]),
    "cfd_half_point_metrics": (C.c_int, [_vp, _i32, _i32, _vp, _vp, _vp]),
    "cfd_lattice_stage_static": (C.c_int, [_vp, _i32, _i32, _i32, _i32, _d, C.POINTER(Params)] + [_vp] * 8),
}


def _header_define(name: str) -> int:
    """An integer #define of include/cfd_rhs.h (the one source of the value)."""
    import re
    text = (pathlib.Path(__file__).resolve().parent.parent / "include" / "cfd_rhs.h").read_text()
    m = re.search(r"^#define\s+" + name + r"\s+(\d+)", text, flags=re.M)
    if not m:
        raise RuntimeError(f"{name} not defined in include/cfd_rhs.h")
    return int(m.group(1))


STATIC_MAX_NODES = _header_define("CFD_STATIC_MAX_NODES")
BATCH_FACE_TILES = _header_define("CFD_BATCH_FACE_TILES")

_lib = None


def load(path: pathlib.Path | None = None):
    """Load the CUDA library (building it first if it is absent)."""
    global _lib
    if _lib is not None:
        return _lib
    p = pathlib.Path(path) if path else LIB_PATH
    if not p.exists():
        _build.build()
    if not p.exists():
        raise RuntimeError(f"libcfd_gb300.so not found at {p}; run build() first")
    lib = C.CDLL(str(p))
    for name, (res, args) in PROTOTYPES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def exported_symbols() -> list[str]:
    return list(PROTOTYPES)
