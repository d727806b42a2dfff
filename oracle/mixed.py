"""CPU restatement of the mixed-precision form (oracle/mixed_oracle.c) driven
like the engine's Step.

TEST INFRASTRUCTURE ONLY: tests/ use it to check the CUDA mixed, batched and
served forms bit for bit.  The product package never imports this module.

MixedOracle keeps the state in an OracleEngine (the FP64 restatement of the
reference), which supplies the binary64 stages the mixed form shares with the
FP64 form -- applyVelocityBC (stencil.go:246-315), computeDivergence
(project.go:42-62), applyPressureBC (project.go:139-163) and subtractGradient
(project.go:172-205) -- and the commit of swept fields (stencil.go:230-235).
The binary32 sweep and the refinement solve come from mixed_oracle.c.  Step
follows aeroflux.go:348-409: velocity BC before each of the six half-step
sweeps x, y, z, z, y, x, a projection after the third and after the sixth.
The projection starts from the last projection's pressure (warm start)
unless warm=False, as the engine does unless AEROFLUX_COLD_START is set.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from .oracle import OracleEngine, lib

FWD, REV = (0, 1, 2), (2, 1, 0)


def _bind():
    L = lib()
    if getattr(L, "_mxo_bound", False):
        return L
    D, F, I64, P = C.c_double, C.c_float, C.c_int64, C.c_void_p
    dp = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
    fp = np.ctypeslib.ndpointer(dtype=np.float32, flags="C_CONTIGUOUS")
    L.mxo_f64_to_f32.argtypes = [D]
    L.mxo_f64_to_f32.restype = F
    L.mxo_f32_to_f64.argtypes = [F]
    L.mxo_f32_to_f64.restype = D
    L.mxo_sweep.argtypes = [I64, I64, I64, I64, C.c_int, F, F, P, P, P, P, P, P]
    L.mxo_sweep.restype = I64
    L.mxo_solver_new.argtypes = [I64, I64, I64, I64, I64, I64, D, D, D, D, D]
    L.mxo_solver_new.restype = P
    L.mxo_solver_free.argtypes = [P]
    L.mxo_solver_free.restype = None
    i32 = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")
    L.mxo_solver_levels.argtypes = [P, i32, i32, i32, i32, i32, i32, fp, fp, fp, C.POINTER(C.c_int32),
                                    C.POINTER(C.c_int32)]
    L.mxo_solver_levels.restype = C.c_int
    L.mxo_refine.argtypes = [P, I64, P, P, I64, C.POINTER(I64), C.POINTER(D)]
    L.mxo_refine.restype = I64
    L.mxo_vcycle.argtypes = [P, fp, fp]
    L.mxo_vcycle.restype = None
    L.mxo_set_mutation.argtypes = [C.c_int]
    L.mxo_set_mutation.restype = None
    del dp
    L._mxo_bound = True
    return L


def f64_to_f32(a: np.ndarray) -> np.ndarray:
    L = _bind()
    return np.array([L.mxo_f64_to_f32(float(x)) for x in np.ravel(a)], dtype=np.float32)


def set_mutation(m: int) -> None:
    """Plant mistake m into the restatement (0: none); see mixed_oracle.h."""
    _bind().mxo_set_mutation(m)


class MixedOracle:
    """aeroflux.New(cfg) of the mixed-precision form, on the CPU."""

    def __init__(self, nx, ny, nz, h, dt, viscosity, density=1.0, ghost=1, div_tol=1e-10, inner_sweeps=2,
                 max_refine=30, vcycles=4, fixed_passes=0, pass_floor=0.0, warm=True, workers=1):
        L = _bind()
        self.o = OracleEngine(nx=nx, ny=ny, nz=nz, ghost=ghost, h=h, dt=dt, viscosity=viscosity, density=density,
                              workers=workers)
        self.nx, self.ny, self.nz, self.g = nx, ny, nz, ghost
        self.h, self.dt, self.nu, self.rho = h, dt, viscosity, density
        self.fixed_passes, self.warm = fixed_passes, warm
        self.s = L.mxo_solver_new(nx, ny, nz, inner_sweeps, max_refine, vcycles, div_tol, dt, density, h,
                                  pass_floor)
        self.passes = 0
        self.vcycles = 0
        self.last_div = 0.0

    def close(self):
        if getattr(self, "s", None):
            _bind().mxo_solver_free(self.s)
            self.s = None
        if getattr(self, "o", None):
            self.o.close()
            self.o = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def data(self, fid: int) -> np.ndarray:
        return self.o.data(fid)

    def levels(self) -> dict:
        n = 16
        a = [np.zeros(n, np.int32) for _ in range(6)]
        w = [np.zeros(n, np.float32) for _ in range(3)]
        tail, cs = C.c_int32(), C.c_int32()
        k = _bind().mxo_solver_levels(self.s, *a, *w, C.byref(tail), C.byref(cs))
        return {"n": k, "dims": [(int(a[0][i]), int(a[1][i]), int(a[2][i])) for i in range(k)],
                "coarsen": [(int(a[3][i]), int(a[4][i]), int(a[5][i])) for i in range(k)],
                "weights": [(float(w[0][i]), float(w[1][i]), float(w[2][i])) for i in range(k)],
                "tail": tail.value, "coarse_sweeps": cs.value}

    def apply_velocity_bc(self):
        self.o.apply_velocity_bc()

    def sweep(self, axis: int, dt: float):
        """One binary32 axis sweep at step dt (dispatch + commit)."""
        inv_h = 1.0 / self.h
        dt_invh = float(np.float32(dt * inv_h))
        lam = float(np.float32(self.nu * dt * inv_h * inv_h))
        u, v, w = (self.o.data(i) for i in (1, 2, 3))
        tu, tv, tw = (self.o.data(i) for i in (5, 6, 7))
        faults = _bind().mxo_sweep(self.nx, self.ny, self.nz, self.g, axis, dt_invh, lam,
                                   *(a.ctypes.data for a in (u, v, w, tu, tv, tw)))
        if faults:
            raise RuntimeError(f"mixed oracle: {faults} NaN backtraces in the axis-{axis} sweep")
        self.o.commit_velocity()

    def project(self):
        """project (project.go:12-34) with the refinement solve."""
        o = self.o
        o.apply_velocity_bc()
        o.compute_divergence()
        p = o.data(0)
        if not self.warm:
            p[:] = 0.0
        h2 = self.h * self.h
        b = np.zeros_like(p)
        g, nx, ny, nz = self.g, self.nx, self.ny, self.nz
        d3 = o.view3(4)
        b3 = b.reshape(d3.shape)
        b3[g:g + nz, g:g + ny, g:g + nx] = h2 * d3[g:g + nz, g:g + ny, g:g + nx]
        vc, ld = C.c_int64(), C.c_double()
        self.passes = _bind().mxo_refine(self.s, g, p.ctypes.data, b.ctypes.data, self.fixed_passes, C.byref(vc),
                                         C.byref(ld))
        self.vcycles, self.last_div = vc.value, ld.value
        o.apply_pressure_bc()
        o.subtract_gradient()
        o.apply_velocity_bc()

    def step(self, n: int = 1):
        half = self.dt * 0.5
        for _ in range(n):
            for k in range(6):
                axis = FWD[k] if k < 3 else REV[k - 3]
                self.o.apply_velocity_bc()
                self.sweep(axis, half)
                if k == 2:
                    self.project()
            self.project()

    def max_divergence(self) -> float:
        return self.o.max_divergence()
