"""Generates tests/golden/oracle_golden.npz: inputs and output digests of the
CPU oracle on small cases.

The reference ships no golden vectors for this path (its tests are property
tests) and Go is unavailable to run it, so these fixtures come from the
oracle, whose own pins are the reference README's published values
(tests/test_oracle_pins.py).  They freeze the oracle's and the CUDA path's
bits: inputs are stored (not regenerated) so libm differences between hosts
cannot move them.  Run from the repository root:

    python tests/golden/make_golden.py
"""
import hashlib
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from aeroflux_gb300 import Config  # noqa: E402
from tests.helpers import FIELDS, oracle_kwargs, seed_arrays  # noqa: E402
from oracle.oracle import OracleEngine  # noqa: E402

CASES = {
    "vortex8": (dict(NX=8, NY=8, NZ=8, H=0.125, DT=0.005), "vortex", 1.0, 3),
    "tg12": (dict(NX=12, NY=12, NZ=12, H=1 / 12, DT=0.004, Viscosity=1e-4, GaussSeidelIters=30), "tg", 1.0, 5),
    "ghost2": (dict(NX=9, NY=6, NZ=11, Ghost=2, H=1 / 11, DT=0.004, Viscosity=5e-4, GaussSeidelIters=10), "tg", 1.0, 3),
    "shear16": (dict(NX=16, NY=16, NZ=16, H=1 / 16, DT=0.004, Viscosity=1e-5, Density=1.0, GaussSeidelIters=60),
                "shear", 1.0, 10),
}
OUT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "oracle_golden.npz")


def digest(a: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(a, dtype="<f8").tobytes()).hexdigest()


def main():
    blob = {}
    for name, (kw, kind, amp, steps) in CASES.items():
        cfg = Config(**kw)
        u, v, w = seed_arrays(cfg, kind, amp)
        with OracleEngine(**oracle_kwargs(cfg)) as o:
            o.data(1)[:] = u
            o.data(2)[:] = v
            o.data(3)[:] = w
            if kind != "shear":
                o.apply_velocity_bc()
            o.step(steps)
            blob[f"{name}/u"], blob[f"{name}/v"], blob[f"{name}/w"] = u, v, w
            blob[f"{name}/steps"] = np.array(steps)
            blob[f"{name}/digests"] = np.array([digest(o.data(i)) for i in range(8)])
            blob[f"{name}/max_divergence"] = np.array(o.max_divergence())
            blob[f"{name}/kinetic_energy"] = np.array(o.kinetic_energy())
    np.savez_compressed(OUT, **blob)
    print(OUT, os.path.getsize(OUT), "bytes;", ", ".join(FIELDS))


if __name__ == "__main__":
    main()
