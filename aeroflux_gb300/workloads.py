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


class Pcg32:
    """PCG32 XSH-RR 64/32 (O'Neill 2014), pcg32_srandom_r seeding."""

    M = (1 << 64) - 1

    def __init__(self, seed: int, stream: int):
        self.state, self.inc = 0, ((stream << 1) | 1) & self.M
        self.next()
        self.state = (self.state + seed) & self.M
        self.next()

    def next(self) -> int:
        old = self.state
        self.state = (old * 6364136223846793005 + self.inc) & self.M
        xs = (((old >> 18) ^ old) >> 27) & 0xFFFFFFFF
        rot = old >> 59
        return ((xs >> rot) | (xs << ((32 - rot) & 31))) & 0xFFFFFFFF

    def uniform(self) -> float:
        a, b = self.next() >> 5, self.next() >> 6
        return (a * 67108864.0 + b) * (1.0 / 9007199254740992.0)

    def choice(self, seq):
        return seq[int(self.uniform() * len(seq))]


def _mixed_instance(rng: Pcg32, dims_choices, div_tol: float = 1e-10) -> Config:
    nx, ny, nz = (rng.choice(dims_choices) for _ in range(3))
    h = 1.0 / max(nx, ny, nz)
    nu = 10.0 ** (-6.0 + 2.0 * rng.uniform())  # log-uniform in [1e-6, 1e-4]
    dt = min(0.004, 0.5 * h * h / (6.0 * nu))
    return Config(NX=nx, NY=ny, NZ=nz, H=h, DT=dt, Viscosity=nu, Density=1.0,
                  Precision=L.AF_PRECISION_MIXED, DivTol=div_tol)


BATCH_DIMS = (32, 48, 64, 96, 128)
BATCH_STEPS = 300


def batched_instances(n: int = 256, seed: int = 42) -> list[Config]:
    """Uneven independent grids: each extent from {32,48,64,96,128}, H=1/max,
    nu log-uniform in [1e-6,1e-4], DT=min(0.004, 0.5 H^2/(6 nu)), mixed form."""
    rng = Pcg32(seed, 0xB47C4)
    return [_mixed_instance(rng, BATCH_DIMS) for _ in range(n)]


SERVE_DIMS = tuple(range(32, 193, 16))


def served_requests(rate: float = 200.0, duration: float = 60.0, seed: int = 42):
    """Poisson arrivals: (arrival time s, Config, steps), extents uniform over
    multiples of 16 in [32,192], steps uniform in [50,500]."""
    rng = Pcg32(seed, 0x5E7E)
    t, out = 0.0, []
    while True:
        import math
        t += -math.log(1.0 - rng.uniform()) / rate
        if t >= duration:
            return out
        cfg = _mixed_instance(rng, SERVE_DIMS)
        steps = 50 + int(rng.uniform() * 451)
        out.append((t, cfg, steps))
