"""Synthetic workloads: the benchmark configurations and their initial fields.

All inputs are synthetic (the reference has no dataset): a Taylor-Green vortex
on the staggered faces plus seeded uniform noise, generated on the host by
af_seed_taylor_green so every consumer sees the same bits.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from . import _lib as L
from .engine import Config


@dataclass(frozen=True)
class Workload:
    name: str
    n: int
    dt: float
    viscosity: float
    steps: int
    gsi: int
    noise: float
    precision: int = L.AF_PRECISION_FP64

    def config(self, **over) -> Config:
        kw = dict(NX=self.n, NY=self.n, NZ=self.n, H=1.0 / self.n, DT=self.dt, Viscosity=self.viscosity,
                  Density=1.0, GaussSeidelIters=self.gsi, Precision=self.precision)
        kw.update(over)
        return Config(**kw)


# Single-grid configurations (H = 1/N, Density = 1, amplitude 1).
PLAIN_64 = Workload("plain-fp64 64^3, DT=0.004, nu=1e-5, GSI=24, 1000 steps, noise 0.01", 64, 0.004, 1e-5, 1000, 24, 0.01)
PLAIN_256 = Workload("plain-fp64 256^3, DT=0.001, nu=1e-5, GSI=200, 200 steps, noise 0.01", 256, 0.001, 1e-5, 200, 200, 0.01)
MIXED_512 = Workload("mixed 512^3, DT=0.0005, nu=1e-5, 100 steps, noise 0.05, div<=1e-10", 512, 0.0005, 1e-5, 100, 200, 0.05,
                     L.AF_PRECISION_MIXED)


def taylor_green(cfg: Config, amp: float = 1.0, noise: float = 0.01, seed: int = 42, stream: int = 0):
    """Padded host arrays (u, v, w) for a normalized cfg."""
    c = Config(**{k: getattr(cfg, k) for k in ("NX", "NY", "NZ", "Ghost", "H", "Viscosity", "Density", "DT",
                                               "Workers", "GaussSeidelIters", "Precision")})
    c.Normalize()
    g = c.Ghost
    cx, cy, cz = c.NX + 2 * g, c.NY + 2 * g, c.NZ + 2 * g
    u = np.empty((cx + 1) * cy * cz)
    v = np.empty(cx * (cy + 1) * cz)
    w = np.empty(cx * cy * (cz + 1))
    rc = L.lib().af_seed_taylor_green(C.byref(c.to_c()), amp, noise, seed, stream,
                                      u.ctypes.data, v.ctypes.data, w.ctypes.data)
    if rc != L.AF_OK:
        raise ValueError("af_seed_taylor_green rejected the configuration")
    return u, v, w
