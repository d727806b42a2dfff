"""Shared helpers: build identical GPU / oracle engines and compare them."""
from __future__ import annotations

import numpy as np

from aeroflux_gb300 import Config, New
from aeroflux_gb300.workloads import taylor_green
from oracle.oracle import OracleEngine

FIELDS = ["P", "U", "V", "W", "Div", "Tmp0", "Tmp1", "Tmp2"]
FID = {n: i for i, n in enumerate(FIELDS)}

_CFG_KEYS = {"NX": "nx", "NY": "ny", "NZ": "nz", "Ghost": "ghost", "H": "h", "Viscosity": "viscosity",
             "Density": "density", "DT": "dt", "Workers": "workers", "GaussSeidelIters": "gauss_seidel_iters"}


def oracle_kwargs(cfg: Config) -> dict:
    return {o: getattr(cfg, k) for k, o in _CFG_KEYS.items()}


def seed_arrays(cfg: Config, kind: str = "tg", amp: float = 1.0, noise: float = 0.01, seed: int = 42):
    """Host (u, v, w) for cfg: 'tg' = Taylor-Green + PCG noise, 'vortex' = the reference's seedVortex."""
    if kind == "tg":
        return taylor_green(cfg, amp, noise, seed)
    with OracleEngine(**oracle_kwargs(cfg)) as o:
        if kind == "vortex":
            o.seed_vortex(amp)
        elif kind == "shear":
            o.seed_shear_layer()
        else:
            raise ValueError(kind)
        return o.data(1).copy(), o.data(2).copy(), o.data(3).copy()


def make_pair(cfg: Config, kind: str = "tg", amp: float = 1.0, noise: float = 0.01, seed: int = 42,
              apply_bc: bool = True, oracle_workers: int | None = None):
    """A GPU engine and an oracle engine holding the same initial field."""
    u, v, w = seed_arrays(cfg, kind, amp, noise, seed)
    gpu = New(cfg)
    gpu.upload("U", u)
    gpu.upload("V", v)
    gpu.upload("W", w)
    kw = oracle_kwargs(cfg)
    if oracle_workers is not None:
        kw["workers"] = oracle_workers
    orc = OracleEngine(**kw)
    orc.data(1)[:] = u
    orc.data(2)[:] = v
    orc.data(3)[:] = w
    if apply_bc and kind != "shear":
        gpu.applyVelocityBC()
        orc.apply_velocity_bc()
    return gpu, orc


def bits(a: np.ndarray) -> np.ndarray:
    return np.ascontiguousarray(a, dtype=np.float64).view(np.uint64)


def same_bits(a: np.ndarray, b: np.ndarray) -> np.ndarray:
    """Element-wise: identical bit patterns, or NaN in both.  NaN payloads
    are platform-defined (the x86 default NaN sets the sign bit, Arm's does
    not, the GPU's canonical NaN differs again), so only NaN-ness is compared."""
    return (bits(a) == bits(b)) | (np.isnan(a) & np.isnan(b))


def assert_bit_identical(gpu, orc, fields=FIELDS, what: str = ""):
    for name in fields:
        g = gpu.download(name)
        o = orc.data(FID[name])
        ok = same_bits(g, o)
        if not ok.all():
            diff = np.nonzero(~ok)[0]
            i = diff[0]
            raise AssertionError(f"{what} field {name}: {diff.size} of {g.size} elements differ; first at {i}: "
                                 f"gpu={g[i]!r} oracle={o[i]!r}")


def max_rel_diff(a: np.ndarray, b: np.ndarray) -> float:
    scale = max(np.max(np.abs(b)), 1e-300)
    return float(np.max(np.abs(a - b)) / scale)
