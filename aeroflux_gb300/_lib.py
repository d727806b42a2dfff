"""ctypes binding of libaeroflux_cuda (include/aeroflux_cuda.h).

The library is built in-tree by aeroflux_gb300/build.py.  There is no CPU
fallback: if the shared library is missing or fails to load, every entry
point raises.
"""
from __future__ import annotations

import ctypes as C
import os
import re

HERE = os.path.dirname(os.path.abspath(__file__))
# AEROFLUX_DEBUG_BOUNDS=1 in the environment selects the bounds-checking
# debug build (libaeroflux_cuda_debug.so, same ABI) for this process.
DEBUG_BOUNDS = os.environ.get("AEROFLUX_DEBUG_BOUNDS", "0") == "1"
LIB_PATH = os.path.join(HERE, "libaeroflux_cuda_debug.so" if DEBUG_BOUNDS else "libaeroflux_cuda.so")
HEADER = os.path.join(os.path.dirname(HERE), "include", "aeroflux_cuda.h")

AF_OK = 0
AF_ERR_CONFIG = -1
AF_ERR_CUDA = -2
AF_ERR_FAULT = -3
AF_ERR_ARG = -4
AF_ERR_UNSUPPORTED = -5
AF_ERR_CLOSED = -6
AF_ERR_NOMEM = -7

AF_PRECISION_FP64 = 0
AF_PRECISION_MIXED = 1

AF_ADVECTION_SEMI_LAGRANGIAN = 0
AF_ADVECTION_MACCORMACK = 1


class AfConfig(C.Structure):
    _fields_ = [
        ("nx", C.c_int64), ("ny", C.c_int64), ("nz", C.c_int64),
        ("ghost", C.c_int64),
        ("h", C.c_double), ("viscosity", C.c_double),
        ("density", C.c_double), ("dt", C.c_double),
        ("workers", C.c_int64), ("gauss_seidel_iters", C.c_int64),
        ("use_sparse_solver", C.c_int32), ("lock", C.c_int32),
        ("precision", C.c_int32), ("device", C.c_int32),
        ("div_tol", C.c_double), ("inner_sweeps", C.c_int64), ("max_refine", C.c_int64),
    ]


class AfStepProfile(C.Structure):
    _fields_ = [("step_ms", C.c_double), ("sweep_ms", C.c_double), ("rbgs_ms", C.c_double),
                ("rbgs_launches", C.c_int64), ("kernel_launches", C.c_int64)]


class AfRequestResult(C.Structure):
    _fields_ = [("id", C.c_int64), ("status", C.c_int32), ("reserved", C.c_int32), ("cells", C.c_int64),
                ("steps", C.c_int64), ("refinement_passes", C.c_int64), ("arrival_s", C.c_double),
                ("admitted_s", C.c_double), ("completed_s", C.c_double), ("max_divergence", C.c_double)]


class AfServerStats(C.Structure):
    _fields_ = [("queued", C.c_int64), ("resident", C.c_int64), ("retained", C.c_int64),
                ("budget_bytes", C.c_int64), ("used_bytes", C.c_int64), ("executed_cell_steps", C.c_int64),
                ("now_s", C.c_double)]


class AfFieldDesc(C.Structure):
    _fields_ = [(n, C.c_int64) for n in ("off", "nx", "ny", "nz", "sy", "sz", "count")]


_E = C.c_void_p
_ERR = (C.c_char_p, C.c_size_t)

# name -> (restype, argtypes); mirrors include/aeroflux_cuda.h one to one.
SIGNATURES = {
    "af_abi_version": (C.c_int, []),
    "af_config_normalize": (C.c_int, [C.POINTER(AfConfig), *_ERR]),
    "af_mac_bytes": (C.c_int64, [C.c_int64] * 4),
    "af_create": (C.c_int, [C.POINTER(AfConfig), C.POINTER(_E), *_ERR]),
    "af_get_config": (C.c_int, [_E, C.POINTER(AfConfig)]),
    "af_field_info": (C.c_int, [_E, C.c_int, C.POINTER(AfFieldDesc)]),
    "af_field_upload": (C.c_int, [_E, C.c_int, C.c_void_p, C.c_size_t]),
    "af_field_download": (C.c_int, [_E, C.c_int, C.c_void_p, C.c_size_t]),
    "af_apply_velocity_bc": (C.c_int, [_E]),
    "af_step": (C.c_int, [_E, C.c_int64]),
    "af_project": (C.c_int, [_E]),
    "af_max_divergence": (C.c_int, [_E, C.POINTER(C.c_double)]),
    "af_kinetic_energy": (C.c_int, [_E, C.POINTER(C.c_double)]),
    "af_max_velocity": (C.c_int, [_E, C.POINTER(C.c_double)]),
    "af_cfl": (C.c_int, [_E, C.POINTER(C.c_double)]),
    "af_enable_sparse_solver": (C.c_int, [_E]),
    "af_enable_multigrid_solver": (C.c_int, [_E, C.c_double]),
    "af_set_advection": (C.c_int, [_E, C.c_int]),
    "af_phase_sweep": (C.c_int, [_E, C.c_int, C.c_double]),
    "af_phase_divergence": (C.c_int, [_E]),
    "af_phase_red_black": (C.c_int, [_E]),
    "af_phase_pressure_bc": (C.c_int, [_E]),
    "af_phase_subtract_gradient": (C.c_int, [_E]),
    "af_last_projection_stats": (C.c_int, [_E, C.POINTER(C.c_int64), C.POINTER(C.c_double)]),
    "af_last_projection_vcycles": (C.c_int, [_E, C.POINTER(C.c_int64)]),
    "af_profile": (C.c_int, [_E, C.c_int]),
    "af_last_step_profile": (C.c_int, [_E, C.POINTER(AfStepProfile)]),
    "af_device_fp64_rate": (C.c_int, [C.c_int, C.POINTER(C.c_double)]),
    "af_selftest_div6": (C.c_int, [C.c_int, C.c_int64, C.c_uint64, C.POINTER(C.c_int64)]),
    "af_selftest_dadd": (C.c_int, [C.c_int, C.c_int64, C.c_uint64, C.POINTER(C.c_int64)]),
    "af_batch_create": (C.c_int, [C.c_int64, C.c_int64, C.c_int32, C.POINTER(_E), *_ERR]),
    "af_batch_slot_bytes": (C.c_int, [C.POINTER(AfConfig), C.POINTER(C.c_int64)]),
    "af_batch_assign": (C.c_int, [_E, C.POINTER(AfConfig), C.POINTER(C.c_int64)]),
    "af_batch_release": (C.c_int, [_E, C.c_int64]),
    "af_batch_set_active": (C.c_int, [_E, C.c_int64, C.c_int]),
    "af_batch_get_config": (C.c_int, [_E, C.c_int64, C.POINTER(AfConfig)]),
    "af_batch_field_info": (C.c_int, [_E, C.c_int64, C.c_int, C.POINTER(AfFieldDesc)]),
    "af_batch_field_upload": (C.c_int, [_E, C.c_int64, C.c_int, C.c_void_p, C.c_size_t]),
    "af_batch_field_download": (C.c_int, [_E, C.c_int64, C.c_int, C.c_void_p, C.c_size_t]),
    "af_batch_apply_velocity_bc": (C.c_int, [_E]),
    "af_batch_step": (C.c_int, [_E, C.c_int64]),
    "af_batch_slot_status": (C.c_int, [_E, C.c_int64, C.POINTER(C.c_int32), *_ERR]),
    "af_batch_max_divergence": (C.c_int, [_E, C.c_int64, C.POINTER(C.c_double)]),
    "af_batch_projection_stats": (C.c_int, [_E, C.c_int64, C.POINTER(C.c_int64), C.POINTER(C.c_double)]),
    "af_batch_tune": (C.c_int, [_E, C.c_int32, *_ERR]),
    "af_batch_profile": (C.c_int, [_E, C.c_int]),
    "af_batch_last_step_profile": (C.c_int, [_E, C.POINTER(AfStepProfile)]),
    "af_batch_seed": (C.c_int, [_E, C.c_int64, C.c_double, C.c_double, C.c_uint64, C.c_uint64]),
    "af_batch_destroy": (None, [_E]),
    "af_server_create": (C.c_int, [C.c_int64, C.c_int64, C.c_int64, C.c_int32, C.c_int32, C.c_int32, C.POINTER(_E),
                                   *_ERR]),
    "af_server_now": (C.c_int, [_E, C.POINTER(C.c_double)]),
    "af_server_submit": (C.c_int, [_E, C.POINTER(AfConfig), C.c_int64, C.c_uint64, C.c_double,
                                   C.POINTER(C.c_int64)]),
    "af_server_round": (C.c_int, [_E, C.POINTER(C.c_int64), C.POINTER(C.c_int64), C.POINTER(C.c_int64)]),
    "af_server_results": (C.c_int, [_E, C.POINTER(AfRequestResult), C.c_int64, C.POINTER(C.c_int64)]),
    "af_server_download": (C.c_int, [_E, C.c_int64, C.c_int, C.c_void_p, C.c_size_t]),
    "af_server_release": (C.c_int, [_E, C.c_int64]),
    "af_server_cancel_queued": (C.c_int, [_E, C.POINTER(C.c_int64)]),
    "af_server_get_stats": (C.c_int, [_E, C.POINTER(AfServerStats)]),
    "af_debug_bounds": (C.c_int, [C.POINTER(C.c_int32), C.POINTER(C.c_uint64), C.POINTER(C.c_uint32), C.c_int32]),
    "af_server_tune": (C.c_int, [_E, C.c_int32, *_ERR]),
    "af_server_destroy": (None, [_E]),
    "af_server_last_error": (C.c_char_p, [_E]),
    "af_batch_last_error": (C.c_char_p, [_E]),
    "af_seed_taylor_green": (C.c_int, [C.POINTER(AfConfig), C.c_double, C.c_double, C.c_uint64, C.c_uint64,
                                       C.c_void_p, C.c_void_p, C.c_void_p]),
    "af_kinetic_energy_noalloc": (C.c_int, [C.POINTER(AfConfig), C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                            C.POINTER(C.c_double), *_ERR]),
    "af_seed_device": (C.c_int, [_E, C.c_double, C.c_double, C.c_uint64, C.c_uint64]),
    "af_close": (C.c_int, [_E]),
    "af_destroy": (None, [_E]),
    "af_last_error": (C.c_char_p, [_E]),
}


def header_symbols() -> list[str]:
    """Every function the public header declares."""
    text = open(HEADER).read()
    return sorted(set(re.findall(r"^\s*(?:[A-Za-z_][\w\s\*]*?)\b(af_\w+)\s*\(", text, re.M)))


_lib = None


def lib() -> C.CDLL:
    """Load the engine library (building it first if it is absent)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            from . import build as _build
            _build.build(debug_bounds=DEBUG_BOUNDS)
        L = C.CDLL(LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def debug_bounds(reset: bool = False) -> tuple[bool, int, int]:
    """(debug build?, first violation record, violations) of the loaded library."""
    en, first, n = C.c_int32(), C.c_uint64(), C.c_uint32()
    rc = lib().af_debug_bounds(C.byref(en), C.byref(first), C.byref(n), int(reset))
    if rc != AF_OK:
        raise RuntimeError(f"af_debug_bounds failed: {rc}")
    return bool(en.value), first.value, n.value
