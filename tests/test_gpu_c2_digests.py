"""The 256^3 plain FP64 workload over its full 200 Steps, against the CPU
oracle's field digests (tests/golden/c2_256_digests.npz, made by
tests/golden/make_c2_digests.py).

Workload: 256^3, H = 1/256, DT = 0.001, Viscosity = 1e-5, 200 red-black
pairs per projection, Taylor-Green amplitude 1 plus uniform +-0.01 PCG32
noise, velocity BC, 200 Steps (aeroflux.go:348-409).  Every field of the
arena (P, U, V, W, Div, Tmp0-2, ghosts included) must match the oracle's
SHA-256 digest after Steps 1, 5, 50, 100 and 200.  Should a digest differ,
the test runs the oracle on this host to that Step and reports the largest
relative difference per field before failing (the bar is bit identity; the
tolerance 1e-12 relative is the fallback the failure message states).
"""
import hashlib
import os

import numpy as np
import pytest

from aeroflux_gb300 import New
from aeroflux_gb300.workloads import PLAIN_256
from tests.golden.tabulated_tg import tabulated_taylor_green
from tests.helpers import FIELDS, max_rel_diff

pytestmark = [pytest.mark.gpu, pytest.mark.slow]

FIXTURE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "c2_256_digests.npz")


def digest(a: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(a, dtype="<f8").tobytes()).hexdigest()


def oracle_fields_at(u, v, w, steps):
    from oracle.oracle import OracleEngine
    with OracleEngine(nx=256, ny=256, nz=256, h=1 / 256, dt=0.001, viscosity=1e-5, density=1.0,
                      gauss_seidel_iters=200, workers=len(os.sched_getaffinity(0))) as o:
        o.data(1)[:] = u
        o.data(2)[:] = v
        o.data(3)[:] = w
        o.apply_velocity_bc()
        o.step(steps)
        return [o.data(i).copy() for i in range(8)]


def test_c2_256_cube_200_steps_match_oracle_digests():
    fx = np.load(FIXTURE)
    u, v, w = tabulated_taylor_green(256, 1, fx["sin"], fx["cos"], 1.0, 0.01, 42, 0)
    assert [digest(a) for a in (u, v, w)] == list(fx["input_digests"]), "input generator differs from the fixture's"
    e = New(PLAIN_256.config())
    for name, a in (("U", u), ("V", v), ("W", w)):
        e.upload(name, a)
    e.applyVelocityBC()
    done = 0
    for k in fx["checkpoints"]:
        e.Step(int(k) - done)
        done = int(k)
        got = [digest(e.download(name)) for name in FIELDS]
        want = list(fx[f"step{k}/digests"])
        bad = [name for name, g, r in zip(FIELDS, got, want) if g != r]
        if bad:
            ref = oracle_fields_at(u, v, w, int(k))
            rel = {name: max_rel_diff(e.download(name), ref[i]) for i, name in enumerate(FIELDS) if name in bad}
            pytest.fail(f"step {k}: digests differ for {bad}; max relative difference {rel} (fallback bar 1e-12)")
        assert e.MaxDivergence() == float(fx[f"step{k}/max_divergence"])
        assert e.MaxVelocity() == float(fx[f"step{k}/max_velocity"])
        print(f"step {k}: all 8 field digests equal the oracle's; max|div| {e.MaxDivergence():.6e}")
    e.Close()
