"""ctypes wrapper of the CPU oracle (oracle/aeroflux_oracle.c).

TEST INFRASTRUCTURE ONLY.  The oracle restates the reference's Go CPU path
(AeroFlex/aeroflux.go, grid.go, stencil.go, project.go) in C; the test suite,
the smoke check and the benchmark's CPU-baseline leg use it as the checker.
The product package never imports this module.

Parity pin status: unpinned at the bit level (no golden vectors exist in the
reference, and Go is unavailable to run it); pinned to the reference's own
property tests and README-published divergence magnitudes.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libaeroflux_oracle.so")

P, U, V, W, DIV, TMP0, TMP1, TMP2 = range(8)
FIELD_NAMES = ["P", "U", "V", "W", "Div", "Tmp0", "Tmp1", "Tmp2"]
AXIS_X, AXIS_Y, AXIS_Z = 0, 1, 2


class OrcConfig(C.Structure):
    _fields_ = [
        ("nx", C.c_int64), ("ny", C.c_int64), ("nz", C.c_int64),
        ("ghost", C.c_int64),
        ("h", C.c_double), ("viscosity", C.c_double),
        ("density", C.c_double), ("dt", C.c_double),
        ("workers", C.c_int64), ("gauss_seidel_iters", C.c_int64),
        ("use_sparse_solver", C.c_int32), ("lock", C.c_int32),
    ]


class OrcField(C.Structure):
    _fields_ = [(n, C.c_int64) for n in ("off", "nx", "ny", "nz", "sy", "sz", "count")]


def _stale() -> bool:
    if not os.path.exists(LIB_PATH):
        return True
    t = os.path.getmtime(LIB_PATH)
    srcs = [f for f in os.listdir(HERE) if f.endswith((".c", ".h")) or f == "Makefile"]
    return any(os.path.getmtime(os.path.join(HERE, f)) > t for f in srcs)


def build(force: bool = False) -> str:
    """Compile the oracle with its Makefile (gcc, -ffp-contract=off)."""
    if force or _stale():
        subprocess.run(["make", "-s", "-B", "-C", HERE, "liboracle"], check=True)
    return LIB_PATH


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(LIB_PATH)
        E = C.c_void_p
        err = (C.c_char_p, C.c_size_t)
        L.orc_normalize.argtypes = [C.POINTER(OrcConfig), *err]
        L.orc_normalize.restype = C.c_int
        L.orc_mac_bytes.argtypes = [C.c_int64] * 4
        L.orc_mac_bytes.restype = C.c_int64
        L.orc_new.argtypes = [C.POINTER(OrcConfig), *err]
        L.orc_new.restype = E
        L.orc_close.argtypes = [E]
        L.orc_close.restype = None
        L.orc_get_config.argtypes = [E, C.POINTER(OrcConfig)]
        L.orc_get_config.restype = None
        L.orc_field_data.argtypes = [E, C.c_int, C.POINTER(OrcField)]
        L.orc_field_data.restype = C.POINTER(C.c_double)
        L.orc_arena.argtypes = [E, C.POINTER(C.c_int64)]
        L.orc_arena.restype = C.POINTER(C.c_uint8)
        for name in ("orc_step", "orc_project"):
            getattr(L, name).argtypes = [E, *err]
            getattr(L, name).restype = C.c_int
        L.orc_sweep.argtypes = [E, C.c_int, C.c_double, *err]
        L.orc_sweep.restype = C.c_int
        for name in ("orc_apply_velocity_bc", "orc_compute_divergence",
                     "orc_solve_pressure_red_black", "orc_apply_pressure_bc",
                     "orc_subtract_gradient", "orc_seed_shear_layer"):
            getattr(L, name).argtypes = [E]
            getattr(L, name).restype = None
        for name in ("orc_max_divergence", "orc_kinetic_energy", "orc_max_velocity", "orc_cfl"):
            getattr(L, name).argtypes = [E]
            getattr(L, name).restype = C.c_double
        L.orc_seed_vortex.argtypes = [E, C.c_double]
        L.orc_seed_vortex.restype = None
        L.orc_commit_velocity.argtypes = [E]
        L.orc_commit_velocity.restype = None
        L.orc_seed_taylor_green.argtypes = [E, C.c_double, C.c_double, C.c_uint64, C.c_uint64]
        L.orc_seed_taylor_green.restype = None
        L.orc_set_advection.argtypes = [E, C.c_int]
        L.orc_set_advection.restype = C.c_int
        L.orc_set_mutation.argtypes = [C.c_int]
        L.orc_set_mutation.restype = None
        L.orc_go_format_float.argtypes = [C.c_double, C.c_char_p, C.c_size_t]
        L.orc_go_format_float.restype = None
        _lib = L
    return _lib


class OracleError(RuntimeError):
    pass


def _cfg(**kw) -> OrcConfig:
    c = OrcConfig()
    for k, v in kw.items():
        setattr(c, k, v)
    return c


def normalize(**kw):
    """Config.Normalize; returns (dict of normalized fields, error string or None)."""
    c = _cfg(**kw)
    buf = C.create_string_buffer(512)
    rc = lib().orc_normalize(C.byref(c), buf, 512)
    out = {n: getattr(c, n) for n, _ in OrcConfig._fields_}
    return out, (buf.value.decode() if rc else None)


def mac_bytes(nx, ny, nz, ghost=1) -> int:
    return lib().orc_mac_bytes(nx, ny, nz, ghost)


def go_format_float(v: float) -> str:
    buf = C.create_string_buffer(64)
    lib().orc_go_format_float(v, buf, 64)
    return buf.value.decode()


class OracleEngine:
    """aeroflux.New(cfg) on the CPU oracle."""

    def __init__(self, **kw):
        c = _cfg(**kw)
        buf = C.create_string_buffer(512)
        h = lib().orc_new(C.byref(c), buf, 512)
        if not h:
            raise OracleError(buf.value.decode())
        self._h = h
        cfg = OrcConfig()
        lib().orc_get_config(h, C.byref(cfg))
        self.cfg = {n: getattr(cfg, n) for n, _ in OrcConfig._fields_}

    def close(self):
        if self._h:
            lib().orc_close(self._h)
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def field(self, fid: int) -> OrcField:
        d = OrcField()
        lib().orc_field_data(self._h, fid, C.byref(d))
        return d

    def data(self, fid: int) -> np.ndarray:
        """Live flat float64 view of the CURRENT descriptor of field fid (like Mesh.Data)."""
        d = OrcField()
        ptr = lib().orc_field_data(self._h, fid, C.byref(d))
        return np.ctypeslib.as_array(ptr, shape=(d.count,))

    def view3(self, fid: int) -> np.ndarray:
        """Live (z, y, x) view of field fid."""
        d = self.field(fid)
        return self.data(fid).reshape(d.nz, d.ny, d.nx)

    def arena(self) -> np.ndarray:
        n = C.c_int64()
        ptr = lib().orc_arena(self._h, C.byref(n))
        return np.ctypeslib.as_array(ptr, shape=(n.value,))

    def _err_call(self, fn, *args):
        buf = C.create_string_buffer(512)
        rc = fn(self._h, *args, buf, 512)
        if rc:
            raise OracleError(buf.value.decode())

    def step(self, n: int = 1):
        for _ in range(n):
            self._err_call(lib().orc_step)

    def project(self):
        self._err_call(lib().orc_project)

    def sweep(self, axis: int, dt: float):
        self._err_call(lib().orc_sweep, axis, dt)

    def set_advection(self, scheme: int):
        """0: the reference's semi-Lagrangian sweeps; 1: MacCormack."""
        if lib().orc_set_advection(self._h, scheme) != 0:
            raise OracleError(f"orc_set_advection({scheme}) failed")

    def commit_velocity(self):
        lib().orc_commit_velocity(self._h)

    def apply_velocity_bc(self):
        lib().orc_apply_velocity_bc(self._h)

    def compute_divergence(self):
        lib().orc_compute_divergence(self._h)

    def solve_pressure_red_black(self):
        lib().orc_solve_pressure_red_black(self._h)

    def apply_pressure_bc(self):
        lib().orc_apply_pressure_bc(self._h)

    def subtract_gradient(self):
        lib().orc_subtract_gradient(self._h)

    def max_divergence(self) -> float:
        return lib().orc_max_divergence(self._h)

    def kinetic_energy(self) -> float:
        return lib().orc_kinetic_energy(self._h)

    def max_velocity(self) -> float:
        return lib().orc_max_velocity(self._h)

    def cfl(self) -> float:
        return lib().orc_cfl(self._h)

    def seed_vortex(self, amp: float = 1.0):
        lib().orc_seed_vortex(self._h, amp)

    def seed_taylor_green(self, amp: float = 1.0, noise: float = 0.01, seed: int = 42, stream: int = 0):
        lib().orc_seed_taylor_green(self._h, amp, noise, seed, stream)

    def seed_shear_layer(self):
        lib().orc_seed_shear_layer(self._h)


def set_mutation(m: int) -> None:
    """Plant mistake m into the oracle (0: none); see aeroflux_oracle.h."""
    lib().orc_set_mutation(m)
