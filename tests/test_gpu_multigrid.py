"""Multigrid projection option of the FP64 engine: the GPU analogue of the
reference's EnableSparseSolver (sparse_darwin.go:26-132, selected in
project.go:19-27), whose semantic is an exact projection.

With it enabled the sweeps stay bit-identical to the oracle, every projection
reaches max|div| <= 1e-12, and whole Steps agree with the oracle's red-black
projection driven to convergence to 1e-10 relative (both are converged
solutions of the same discrete problem).
"""
import math

import numpy as np
import pytest

from aeroflux_gb300 import AF_PRECISION_MIXED, AerofluxError, Config, New
from aeroflux_gb300.engine import FaultError
from oracle.oracle import OracleError
from tests.helpers import FID, assert_bit_identical, make_pair, max_rel_diff

pytestmark = pytest.mark.gpu


def cfg(n, **kw):
    base = dict(NX=n[0], NY=n[1], NZ=n[2], H=1.0 / max(n), DT=0.004, Viscosity=1e-5, Density=1.0)
    base.update(kw)
    return Config(**base)


@pytest.mark.parametrize("n", [(16, 16, 16), (24, 20, 18), (33, 17, 20), (64, 64, 64), (48, 32, 96)])
def test_projection_reaches_1e12_or_the_roundoff_floor(n):
    c = cfg(n)
    gpu, orc = make_pair(c, "tg", 1.0, 0.01)
    gpu.EnableMultigridSolver()
    before = gpu.MaxDivergence()
    gpu.project()
    passes, _ = gpu.LastProjectionStats()
    md = gpu.MaxDivergence()
    # Round-off floor of the binary64 residual: |B| = h^2 |Div| = h*rho/DT *
    # max|div u| (before), times a few ulps, times DT/(rho h^2).
    floor = 8 * 2.0 ** -53 * before / c.H
    print(f"{n}: max|div| {before:.3e} -> {md:.3e} in {passes} passes (floor {floor:.1e})")
    assert md <= max(1e-12, floor)
    assert 1 <= passes < 20  # stopped at the tolerance or the floor, not at the pass cap
    gpu.Close()
    orc.close()


def test_sweeps_stay_bit_exact():
    gpu, orc = make_pair(cfg((12, 10, 9)), "tg", 1.0, 0.01)
    gpu.EnableMultigridSolver()
    dt = orc.cfg["dt"] * 0.5
    for axis in (0, 1, 2):
        gpu.sweep(axis, dt)
        orc.sweep(axis, dt)
    assert_bit_identical(gpu, orc, ["U", "V", "W", "Tmp0", "Tmp1", "Tmp2"], "sweeps with multigrid enabled")
    orc.close()


def test_steps_match_converged_oracle():
    n, steps = (16, 16, 16), 5
    gpu, orc = make_pair(cfg(n, GaussSeidelIters=4000), "tg", 1.0, 0.01)
    gpu.EnableMultigridSolver()
    gpu.Step(steps)
    orc.step(steps)
    assert gpu.MaxDivergence() <= 1e-12
    assert orc.max_divergence() < 1e-11
    for name in ("U", "V", "W"):
        rel = max_rel_diff(gpu.download(name), orc.data(FID[name]))
        print(f"{steps} steps {name}: max|diff|/max|ref| = {rel:.2e}")
        assert rel < 1e-10
    orc.close()


def test_every_step_reaches_1e12_and_repeats_bit_for_bit():
    outs = []
    for _ in range(2):
        e = New(cfg((40, 24, 32)))
        e.SeedDevice(1.0, 0.01, 42, 3)
        e.applyVelocityBC()
        e.EnableMultigridSolver()
        for _ in range(3):
            e.Step()
            assert e.MaxDivergence() <= 1e-12
        outs.append(np.concatenate([e.download(k).view(np.uint64) for k in ("U", "V", "W", "P")]))
        e.Close()
    assert np.array_equal(outs[0], outs[1])


def test_custom_tolerance_and_idempotence():
    gpu, orc = make_pair(cfg((32, 32, 32)), "tg", 1.0, 0.01)
    gpu.EnableMultigridSolver(1e-6)
    gpu.EnableMultigridSolver(1e-12)  # already enabled: no change, like EnableSparseSolver
    gpu.project()
    md = gpu.MaxDivergence()
    assert md <= 1e-6
    assert md > 1e-12  # the first tolerance stands
    with pytest.raises(AerofluxError) as ex:
        gpu.EnableSparseSolver()  # the reference's non-Darwin answer is unchanged
    assert str(ex.value).startswith("aeroflux: sparse direct solver requires darwin")
    orc.close()


def test_rejected_for_mixed_form_and_bad_tolerance():
    e = New(cfg((16, 16, 16), Precision=AF_PRECISION_MIXED))
    with pytest.raises(AerofluxError):
        e.EnableMultigridSolver()
    e.Close()
    e = New(cfg((16, 16, 16)))
    for bad in (-1.0, math.inf, math.nan):
        with pytest.raises(AerofluxError):
            e.EnableMultigridSolver(bad)
    e.Close()


def test_nan_fault_message_and_state_match_oracle():
    c = Config(NX=8, NY=8, NZ=8, H=0.125, DT=0.005)
    gpu, orc = make_pair(c, "vortex", 1.0, oracle_workers=1)
    gpu.EnableMultigridSolver()
    f = orc.field(FID["U"])
    idx = 4 + 4 * f.sy + 4 * f.sz
    a = gpu.download("U")
    a[idx] = math.nan
    gpu.upload("U", a)
    orc.data(FID["U"])[idx] = math.nan
    with pytest.raises(OracleError) as oex:
        orc.step()
    with pytest.raises(FaultError) as gex:
        gpu.Step()
    assert str(gex.value) == str(oex.value)
    # The fault comes in the first sweep, before any projection: the state
    # matches the oracle's bit for bit.
    assert_bit_identical(gpu, orc, ["U", "V", "W", "P", "Div"], "state after fault")
    orc.close()
