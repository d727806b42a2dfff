"""Generates tests/golden/c2_256_digests.npz: the CPU oracle's SHA-256 field
digests over 200 Steps of the 256^3 plain FP64 workload.

TEST INFRASTRUCTURE.  Workload: 256^3 MAC grid, H = 1/256, DT = 0.001,
Viscosity = 1e-5, Density = 1, 200 red-black pairs per projection
(GaussSeidelIters), Taylor-Green amplitude 1 plus uniform +-0.01 PCG32 noise
(seed 42, stream 0), the velocity BC applied, then 200 Steps
(aeroflux.go:348-409).  The initial field comes from tabulated_tg.py, whose
sin/cos tables are stored here so the input is bit-identical on any host.

The oracle runs with every host core (its results do not depend on the
worker count).  It takes about a quarter of an hour on 8 x86 cores.  Run
from the repository root:

    python tests/golden/make_c2_digests.py
"""
from __future__ import annotations

import hashlib
import os
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from oracle.oracle import OracleEngine  # noqa: E402
from tests.golden.tabulated_tg import tabulated_taylor_green, trig_tables  # noqa: E402

N, DT, NU, GSI, STEPS = 256, 0.001, 1e-5, 200, 200
CHECKPOINTS = (1, 5, 50, 100, 200)
OUT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "c2_256_digests.npz")


def digest(a: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(a, dtype="<f8").tobytes()).hexdigest()


def main():
    sin_t, cos_t = trig_tables(N)
    u, v, w = tabulated_taylor_green(N, 1, sin_t, cos_t, 1.0, 0.01, 42, 0)
    blob = {"sin": sin_t, "cos": cos_t, "input_digests": np.array([digest(u), digest(v), digest(w)]),
            "checkpoints": np.array(CHECKPOINTS)}
    workers = len(os.sched_getaffinity(0))
    with OracleEngine(nx=N, ny=N, nz=N, h=1.0 / N, dt=DT, viscosity=NU, density=1.0, gauss_seidel_iters=GSI,
                      workers=workers) as o:
        o.data(1)[:] = u
        o.data(2)[:] = v
        o.data(3)[:] = w
        o.apply_velocity_bc()
        t0 = time.time()
        done = 0
        for k in CHECKPOINTS:
            o.step(k - done)
            done = k
            blob[f"step{k}/digests"] = np.array([digest(o.data(i)) for i in range(8)])
            blob[f"step{k}/max_divergence"] = np.array(o.max_divergence())
            blob[f"step{k}/max_velocity"] = np.array(o.max_velocity())
            print(f"step {k}: max|div| {o.max_divergence():.6e}, {time.time() - t0:.0f} s", flush=True)
    np.savez_compressed(OUT, **blob)
    print(OUT, os.path.getsize(OUT), "bytes")


if __name__ == "__main__":
    main()
