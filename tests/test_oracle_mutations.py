"""Self-checks of the oracles, on the CPU.

The reference ships no golden vectors for this path, so the bit-level parity
tests rest on the restatements.  These tests show that those comparisons are
sharp: each planted mistake -- a swapped boundary loop (stencil.go:279-290),
a contracted multiply-add, a swapped colour order (project.go:88-97), a
reordered pressure BC (project.go:139-163), a re-paired neighbour sum
(project.go:125), and the same kinds of mistakes in the binary32
restatement -- changes the bits the parity tests compare.  They also pin the
binary32 restatement's own rules (conversion rounding, convergence, the
multigrid hierarchy).
"""
import numpy as np
import pytest

from aeroflux_gb300 import Config
from aeroflux_gb300.workloads import taylor_green
from oracle import mixed as mx
from oracle import oracle as fp
from oracle.mixed import MixedOracle
from oracle.oracle import OracleEngine
from tests.helpers import same_bits


def fp64_run(mutation, n=(14, 12, 10), steps=2):
    nx, ny, nz = n
    cfg = Config(NX=nx, NY=ny, NZ=nz, H=1 / nx, DT=0.004, Viscosity=1e-4, GaussSeidelIters=6)
    u, v, w = taylor_green(cfg, 1.0, 0.01)
    rng = np.random.default_rng(3)
    fp.set_mutation(mutation)
    try:
        with OracleEngine(nx=nx, ny=ny, nz=nz, h=1 / nx, dt=0.004, viscosity=1e-4, density=1.0,
                          gauss_seidel_iters=6) as o:
            for i, a in ((1, u), (2, v), (3, w)):
                a = a.copy()
                ghost = a == 0.0
                a[ghost] = rng.uniform(-1, 1, int(ghost.sum()))
                o.data(i)[:] = a
            o.apply_velocity_bc()
            o.step(steps)
            return [o.data(i).copy() for i in range(8)]
    finally:
        fp.set_mutation(0)


def mixed_run(mutation, n=(24, 20, 18), steps=1):
    nx, ny, nz = n
    cfg = Config(NX=nx, NY=ny, NZ=nz, H=1 / max(n), DT=0.004, Viscosity=1e-4)
    u, v, w = taylor_green(cfg, 1.0, 0.01)
    mx.set_mutation(mutation)
    try:
        with MixedOracle(nx, ny, nz, 1 / max(n), 0.004, 1e-4) as o:
            for i, a in ((1, u), (2, v), (3, w)):
                o.data(i)[:] = a
            o.apply_velocity_bc()
            o.step(steps)
            return [o.data(i).copy() for i in range(8)]
    finally:
        mx.set_mutation(0)


def differs(a, b):
    return any(not same_bits(x, y).all() for x, y in zip(a, b))


def test_fp64_oracle_is_deterministic():
    assert not differs(fp64_run(0), fp64_run(0))


@pytest.mark.parametrize("mutation", [1, 2, 3, 4, 5])
def test_fp64_mutations_change_the_bits(mutation):
    assert differs(fp64_run(0), fp64_run(mutation))


def test_mixed_oracle_is_deterministic():
    assert not differs(mixed_run(0), mixed_run(0))


@pytest.mark.parametrize("mutation,n", [(1, (24, 20, 18)), (2, (24, 20, 18)), (3, (24, 20, 18)), (4, (40, 1, 1))])
def test_mixed_mutations_change_the_bits(mutation, n):
    assert differs(mixed_run(0, n), mixed_run(mutation, n))


def test_binary32_conversion_rounds_half_away_and_flushes():
    rng = np.random.default_rng(1)
    x = rng.standard_normal(2000) * 10.0 ** rng.integers(-30, 30, 2000)
    got = mx.f64_to_f32(x)
    # Off the ties, round-half-away equals numpy's round-half-even.
    assert np.array_equal(got, x.astype(np.float32))
    one = 1.0 + 2.0 ** -24  # exactly halfway between 1 and the next binary32
    assert mx.f64_to_f32(np.array([one, -one])).tolist() == [1.0000001192092896, -1.0000001192092896]
    tiny = np.array([1e-39, -1e-39, 1e-300])  # below FLT_MIN: signed zero
    out = mx.f64_to_f32(tiny)
    assert np.all(out == 0) and np.signbit(out).tolist() == [False, True, False]
    assert np.isinf(mx.f64_to_f32(np.array([1e300]))[0])


@pytest.mark.parametrize("n", [(16, 16, 16), (33, 17, 20), (40, 1, 1), (3, 2, 5)])
def test_mixed_oracle_projection_reaches_tolerance(n):
    nx, ny, nz = n
    cfg = Config(NX=nx, NY=ny, NZ=nz, H=1 / max(n), DT=0.004, Viscosity=1e-5)
    u, v, w = taylor_green(cfg, 1.0, 0.01)
    with MixedOracle(nx, ny, nz, 1 / max(n), 0.004, 1e-5) as o:
        for i, a in ((1, u), (2, v), (3, w)):
            o.data(i)[:] = a
        o.apply_velocity_bc()
        o.project()
        assert o.max_divergence() <= 1e-10


def test_mixed_oracle_hierarchy():
    with MixedOracle(48, 32, 96, 1 / 96, 0.004, 1e-5) as o:
        lv = o.levels()
    # Semi-coarsening keeps the operator's anisotropy in binary32 weights.
    assert lv["dims"][:4] == [(48, 32, 96), (24, 16, 48), (12, 8, 24), (6, 4, 12)]
    assert lv["weights"][1] == (0.25, 0.25, 0.25)
    d = lv["dims"][-1]
    assert d[0] * d[1] * d[2] <= 8 or lv["coarsen"][-1] == (0, 0, 0)
    with MixedOracle(40, 1, 1, 1 / 40, 0.004, 1e-5) as o:
        lv = o.levels()
    assert all(w[1] == 0.0 and w[2] == 0.0 for w in lv["weights"])
