"""Host-side mirror of the reference's Go API over the C ABI.

Names and semantics follow package aeroflux (AeroFlex/aeroflux.go, grid.go):

    e = New(Config(NX=64, NY=64, NZ=64, H=1/64, DT=0.004, Viscosity=1e-5))
    u = e.Mesh.Data(e.Mesh.U)     # padded float64 view of U (grid.go:147)
    u[...] = seed                 # callers write the initial state into views
    e.Step()                      # aeroflux.go:348
    e.MaxDivergence()             # project.go:210
    e.Close()                     # aeroflux.go:419

The fields live in device memory.  Mesh.Data returns a host mirror of the
whole padded field; the engine uploads every outstanding mirror before its
next device operation and refreshes them afterwards, so writes and reads
through a view behave like the reference's aliasing slices.  Mesh.Release()
drops the mirrors (the bulk path uses upload/download directly).

Errors are raised as AerofluxError carrying the reference's message;
contained faults raise FaultError (a subclass).
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field, fields as dc_fields

import numpy as np

from . import _lib as L


class AerofluxError(RuntimeError):
    """An error returned by the engine; str() is the reference's message."""

    def __init__(self, msg: str, code: int = L.AF_ERR_CONFIG):
        super().__init__(msg)
        self.code = code


class FaultError(AerofluxError):
    """A contained fault ("aeroflux: guard-page fault contained: ...")."""


@dataclass
class Config:
    """Config, aeroflux.go:14-41, plus the GB300 extensions of af_config."""

    NX: int = 0
    NY: int = 0
    NZ: int = 0
    Ghost: int = 0
    H: float = 0.0
    Viscosity: float = 0.0
    Density: float = 0.0
    DT: float = 0.0
    Workers: int = 0
    GaussSeidelIters: int = 0
    UseSparseSolver: bool = False
    Lock: bool = False
    # extensions
    Precision: int = L.AF_PRECISION_FP64
    DivTol: float = 0.0
    InnerSweeps: int = 0
    MaxRefine: int = 0
    Device: int = 0

    _MAP = (("NX", "nx"), ("NY", "ny"), ("NZ", "nz"), ("Ghost", "ghost"), ("H", "h"),
            ("Viscosity", "viscosity"), ("Density", "density"), ("DT", "dt"), ("Workers", "workers"),
            ("GaussSeidelIters", "gauss_seidel_iters"), ("UseSparseSolver", "use_sparse_solver"),
            ("Lock", "lock"), ("Precision", "precision"), ("DivTol", "div_tol"),
            ("InnerSweeps", "inner_sweeps"), ("MaxRefine", "max_refine"), ("Device", "device"))

    def to_c(self) -> L.AfConfig:
        c = L.AfConfig()
        for py, cn in self._MAP:
            v = getattr(self, py)
            setattr(c, cn, int(v) if isinstance(v, bool) else v)
        return c

    @classmethod
    def from_c(cls, c: L.AfConfig) -> "Config":
        out = cls()
        for py, cn in cls._MAP:
            v = getattr(c, cn)
            setattr(out, py, bool(v) if py in ("UseSparseSolver", "Lock") else v)
        return out

    def Normalize(self) -> None:
        """(*Config).Normalize, aeroflux.go:47-113: fills defaults in place or raises."""
        c = self.to_c()
        buf = C.create_string_buffer(512)
        rc = L.lib().af_config_normalize(C.byref(c), buf, 512)
        if rc != L.AF_OK:
            raise AerofluxError(buf.value.decode(), rc)
        for py, cn in self._MAP:
            v = getattr(c, cn)
            setattr(self, py, bool(v) if py in ("UseSparseSolver", "Lock") else v)


FIELD_IDS = {"P": 0, "U": 1, "V": 2, "W": 3, "Div": 4, "Tmp0": 5, "Tmp1": 6, "Tmp2": 7}


@dataclass(frozen=True)
class Field:
    """Field, grid.go:12-31."""

    Off: int
    NX: int
    NY: int
    NZ: int
    SY: int
    SZ: int
    Count: int
    name: str = field(default="", compare=False)

    def Index(self, x: int, y: int, z: int) -> int:
        return x + y * self.SY + z * self.SZ


class Mesh:
    """MAC, grid.go:52-73: geometry and host-mirror views of the device fields."""

    def __init__(self, eng: "Engine"):
        self._e = eng
        c = eng.Cfg
        self.NX, self.NY, self.NZ, self.Ghost, self.H = c.NX, c.NY, c.NZ, c.Ghost, c.H
        self.Bytes = L.lib().af_mac_bytes(c.NX, c.NY, c.NZ, c.Ghost)
        self._views: dict[int, np.ndarray] = {}

    def _desc(self, name: str) -> Field:
        d = L.AfFieldDesc()
        rc = L.lib().af_field_info(self._e._h, FIELD_IDS[name], C.byref(d))
        if rc != L.AF_OK:
            raise AerofluxError("aeroflux: field info failed", rc)
        return Field(d.off, d.nx, d.ny, d.nz, d.sy, d.sz, d.count, name)

    P = property(lambda s: s._desc("P"))
    U = property(lambda s: s._desc("U"))
    V = property(lambda s: s._desc("V"))
    W = property(lambda s: s._desc("W"))
    Div = property(lambda s: s._desc("Div"))
    Tmp0 = property(lambda s: s._desc("Tmp0"))
    Tmp1 = property(lambda s: s._desc("Tmp1"))
    Tmp2 = property(lambda s: s._desc("Tmp2"))

    def Data(self, f: Field) -> np.ndarray:
        """Mesh.Data(&f), grid.go:147-149: a flat float64 view of field f."""
        fid = FIELD_IDS[f.name]
        v = self._views.get(fid)
        if v is None:
            v = np.empty(f.Count, dtype=np.float64)
            self._e._download(fid, v)
            self._views[fid] = v
        return v

    def CellIndex(self, i: int, j: int, k: int) -> int:
        return i + j * self.NX + k * self.NX * self.NY

    def Release(self) -> None:
        """Push any edits and drop every host mirror."""
        self._push()
        self._views.clear()

    def _push(self) -> None:
        for fid, v in self._views.items():
            self._e._upload(fid, v)

    def _pull(self) -> None:
        for fid, v in self._views.items():
            self._e._download(fid, v)


class Engine:
    """Engine, aeroflux.go:133-172, backed by one libaeroflux_cuda engine."""

    def __init__(self, cfg: Config):
        c = cfg.to_c()
        h = C.c_void_p()
        buf = C.create_string_buffer(512)
        rc = L.lib().af_create(C.byref(c), C.byref(h), buf, 512)
        if rc != L.AF_OK:
            raise AerofluxError(buf.value.decode(), rc)
        self._h = h
        out = L.AfConfig()
        L.lib().af_get_config(self._h, C.byref(out))
        self.Cfg = Config.from_c(out)
        self.Mesh = Mesh(self)

    # --- plumbing -----------------------------------------------------------
    def _check(self, rc: int) -> None:
        if rc == L.AF_OK:
            return
        msg = (L.lib().af_last_error(self._h) or b"").decode()
        raise (FaultError if rc == L.AF_ERR_FAULT else AerofluxError)(msg, rc)

    def _upload(self, fid: int, arr: np.ndarray) -> None:
        a = np.ascontiguousarray(arr, dtype=np.float64)
        self._check(L.lib().af_field_upload(self._h, fid, a.ctypes.data, a.size))

    def _download(self, fid: int, arr: np.ndarray) -> None:
        assert arr.flags.c_contiguous and arr.dtype == np.float64
        self._check(L.lib().af_field_download(self._h, fid, arr.ctypes.data, arr.size))

    def _device_op(self, fn, *args) -> None:
        self.Mesh._push()
        try:
            self._check(fn(self._h, *args))
        finally:
            self.Mesh._pull()

    def _scalar(self, fn) -> float:
        self.Mesh._push()
        out = C.c_double()
        self._check(fn(self._h, C.byref(out)))
        return out.value

    # --- reference API --------------------------------------------------------
    def Step(self, n: int = 1) -> None:
        """(*Engine).Step, aeroflux.go:348-409 (n steps; stops at the first fault)."""
        self._device_op(L.lib().af_step, n)

    def MaxDivergence(self) -> float:
        return self._scalar(L.lib().af_max_divergence)

    def KineticEnergy(self) -> float:
        return self._scalar(L.lib().af_kinetic_energy)

    def MaxVelocity(self) -> float:
        return self._scalar(L.lib().af_max_velocity)

    def CFL(self) -> float:
        return self._scalar(L.lib().af_cfl)

    def EnableSparseSolver(self) -> None:
        self._check(L.lib().af_enable_sparse_solver(self._h))

    def EnableMultigridSolver(self, div_tol: float = 0.0) -> None:
        """The GPU analogue of EnableSparseSolver (sparse_darwin.go:26-132):
        projections solve to max|div| <= div_tol (0: 1e-12) by binary64
        refinement around binary32 multigrid; the sweeps stay bit-exact."""
        self._check(L.lib().af_enable_multigrid_solver(self._h, div_tol))

    def SetAdvection(self, scheme: int) -> None:
        """AF_ADVECTION_SEMI_LAGRANGIAN (the reference's, bit-exact) or
        AF_ADVECTION_MACCORMACK (limited MacCormack, FP64 form only)."""
        self._check(L.lib().af_set_advection(self._h, scheme))

    def Close(self) -> None:
        """(*Engine).Close, aeroflux.go:419-439; idempotent."""
        if self._h:
            L.lib().af_destroy(self._h)
            self._h = None
            self.Mesh._views.clear()

    # --- the reference's unexported methods its tests call --------------------
    def project(self) -> None:
        self._device_op(L.lib().af_project)

    def applyVelocityBC(self) -> None:
        self._device_op(L.lib().af_apply_velocity_bc)

    # --- phase hooks for stage-level tests -----------------------------------
    def sweep(self, axis: int, dt: float) -> None:
        self._device_op(L.lib().af_phase_sweep, axis, dt)

    def computeDivergence(self) -> None:
        self._device_op(L.lib().af_phase_divergence)

    def solvePressureRedBlack(self) -> None:
        self._device_op(L.lib().af_phase_red_black)

    def applyPressureBC(self) -> None:
        self._device_op(L.lib().af_phase_pressure_bc)

    def subtractGradient(self) -> None:
        self._device_op(L.lib().af_phase_subtract_gradient)

    def Profile(self, enable: bool = True) -> None:
        """Carry event nodes in the step graph (device time per stage)."""
        self._check(L.lib().af_profile(self._h, int(enable)))

    def LastStepProfile(self) -> L.AfStepProfile:
        out = L.AfStepProfile()
        self._check(L.lib().af_last_step_profile(self._h, C.byref(out)))
        return out

    def LastProjectionStats(self) -> tuple[int, float]:
        passes = C.c_int64()
        md = C.c_double()
        self._check(L.lib().af_last_projection_stats(self._h, C.byref(passes), C.byref(md)))
        return passes.value, md.value

    def LastProjectionVCycles(self) -> int:
        v = C.c_int64()
        self._check(L.lib().af_last_projection_vcycles(self._h, C.byref(v)))
        return v.value

    def SeedDevice(self, amp: float = 1.0, noise: float = 0.01, seed: int = 42, stream: int = 0) -> None:
        """Device-side Taylor-Green + PCG32 initial field (apply the BC after)."""
        self._device_op(L.lib().af_seed_device, amp, noise, seed, stream)

    # --- bulk transfer (no mirrors) ------------------------------------------
    def upload(self, name: str, arr: np.ndarray) -> None:
        self._upload(FIELD_IDS[name], arr)

    def download(self, name: str, out: np.ndarray | None = None) -> np.ndarray:
        f = self.Mesh._desc(name)
        if out is None:
            out = np.empty(f.Count, dtype=np.float64)
        self._download(FIELD_IDS[name], out)
        return out

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.Close()

    def __del__(self):
        try:
            self.Close()
        except Exception:
            pass


def New(cfg: Config) -> Engine:
    """aeroflux.New, aeroflux.go:176-213."""
    return Engine(cfg)


def MACBytes(nx: int, ny: int, nz: int, ghost: int) -> int:
    """MACBytes, grid.go:138-144."""
    return L.lib().af_mac_bytes(nx, ny, nz, ghost)
