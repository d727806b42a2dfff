"""The benchmark configurations, checked at their own sizes.

- 64^3, DT=0.004, nu=1e-5, GSI=24, 1000 Steps (the CPU-runnable case): the
  CUDA path must equal the oracle bit for bit after all 1000 steps; the test
  reports MaxDivergence and the per-field max|diff|/max|ref| (zero).
- 256^3, DT=0.001, nu=1e-5, GSI=200 (the benchmark workload): five Steps
  bit-identical to the oracle at full size, then size-independent properties
  over the configuration's 200 Steps (finite fields, no-slip walls exactly
  zero, the run reproducible bit for bit).
"""
import numpy as np
import pytest

from aeroflux_gb300 import New
from aeroflux_gb300.workloads import PLAIN_256, PLAIN_64, taylor_green
from tests.helpers import FIELDS, assert_bit_identical, bits, make_pair, max_rel_diff

pytestmark = [pytest.mark.gpu, pytest.mark.slow]


def test_plain_64_cube_1000_steps_bit_exact():
    cfg = PLAIN_64.config()
    gpu, orc = make_pair(cfg, "tg", 1.0, PLAIN_64.noise)
    gpu.Step(PLAIN_64.steps)
    orc.step(PLAIN_64.steps)
    assert_bit_identical(gpu, orc, FIELDS, "64^3 after 1000 steps")
    md_g, md_o = gpu.MaxDivergence(), orc.max_divergence()
    assert md_g == md_o
    rel = {n: max_rel_diff(gpu.download(n), orc.data(i)) for i, n in enumerate(FIELDS) if n in ("U", "V", "W", "P")}
    print(f"64^3 x1000: max|div|={md_g:.6e}; max|diff|/max|ref| per field: {rel}")
    assert all(r == 0.0 for r in rel.values())


def test_plain_256_cube_steps_bit_exact_at_full_size():
    cfg = PLAIN_256.config()
    gpu, orc = make_pair(cfg, "tg", 1.0, PLAIN_256.noise)
    for k in range(1, 6):
        gpu.Step(1)
        orc.step(1)
        assert_bit_identical(gpu, orc, ["U", "V", "W", "P", "Div"], f"256^3 after {k} steps")
        assert gpu.MaxDivergence() == orc.max_divergence()


def test_plain_256_cube_properties_over_steps():
    cfg = PLAIN_256.config()
    runs = []
    for _ in range(2):
        e = New(cfg)
        u, v, w = taylor_green(e.Cfg, 1.0, PLAIN_256.noise)
        for n, a in (("U", u), ("V", v), ("W", w)):
            e.upload(n, a)
        e.applyVelocityBC()
        e.Step(PLAIN_256.steps)
        print(f"256^3 x {PLAIN_256.steps}: max|div| {e.MaxDivergence():.6e}, KE {e.KineticEnergy():.6e}")
        U = e.download("U")
        for n in ("U", "V", "W", "P"):
            assert np.all(np.isfinite(e.download(n)))
        u3 = U.reshape(258, 258, 259)
        assert np.all(u3[1:257, 1:257, 1] == 0) and np.all(u3[1:257, 1:257, 257] == 0)
        runs.append(bits(U).copy())
        e.Close()
    assert np.array_equal(runs[0], runs[1])
