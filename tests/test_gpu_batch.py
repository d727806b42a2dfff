"""Batched form: many mixed-precision grids of uneven sizes in one batch.

Each slot must compute exactly the bits it computes alone (an af_create'd
MIXED engine), under any tuned launch shapes, while slots come and go
between steps, and a fault in one slot must not touch the others.
"""
import math

import numpy as np
import pytest

from aeroflux_gb300 import AF_PRECISION_MIXED, AerofluxError, Config, New
from aeroflux_gb300.batch import Batch
from aeroflux_gb300.workloads import batched_instances, taylor_green
from tests.helpers import bits

pytestmark = pytest.mark.gpu

FIELDS4 = ("U", "V", "W", "P")


def cfg(nx, ny, nz, nu=1e-5, dt=0.002):
    h = 1.0 / max(nx, ny, nz)
    return Config(NX=nx, NY=ny, NZ=nz, H=h, DT=min(dt, 0.5 * h * h / (6 * nu)), Viscosity=nu, Density=1.0,
                  Precision=AF_PRECISION_MIXED, DivTol=1e-10)


SHAPES = [cfg(16, 16, 16), cfg(32, 48, 24, 3e-5), cfg(20, 12, 36, 1e-4), cfg(33, 17, 20), cfg(64, 32, 16, 1e-6),
          cfg(24, 24, 96, 5e-6)]


def seed_fields(c, stream):
    return taylor_green(c, 1.0, 0.01, 42, stream)


def alone(c, stream, steps):
    e = New(c)
    for n, a in zip(("U", "V", "W"), seed_fields(e.Cfg, stream)):
        e.upload(n, a)
    e.applyVelocityBC()
    e.Step(steps)
    out = {n: e.download(n) for n in FIELDS4}
    e.Close()
    return out


def batched(cfgs, steps, tune=False):
    b = Batch(len(cfgs))
    slots = [b.assign(c) for c in cfgs]
    if tune:
        b.tune(3)
    for s, c in zip(slots, cfgs):
        for n, a in zip(("U", "V", "W"), seed_fields(b.config(s), s)):
            b.upload(s, n, a)
    b.apply_velocity_bc()
    b.step(steps)
    out = [{n: b.download(s, n) for n in FIELDS4} for s in slots]
    divs = [b.max_divergence(s) for s in slots]
    b.close()
    return out, divs


def test_each_slot_is_bit_identical_to_its_grid_alone():
    steps = 3
    got, divs = batched(SHAPES, steps)
    for s, c in enumerate(SHAPES):
        ref = alone(c, s, steps)
        for n in FIELDS4:
            assert np.array_equal(bits(got[s][n]), bits(ref[n])), f"slot {s} field {n}"
        assert divs[s] <= 1e-10


def test_slot_with_odd_sweeps_in_an_even_batch_converges():
    # The batch sweeps as often as its first slot; a slot whose own count
    # has the other parity smooths in place instead of in fused pairs.
    a = Config(**{**cfg(32, 32, 32).__dict__, "InnerSweeps": 2})
    b_ = Config(**{**cfg(48, 24, 32).__dict__, "InnerSweeps": 3})
    _, divs = batched([a, b_], 2)
    assert max(divs) <= 1e-10


def test_tuned_launch_shapes_do_not_change_results():
    a, _ = batched(SHAPES[:4], 2, tune=False)
    b, _ = batched(SHAPES[:4], 2, tune=True)
    for s in range(4):
        for n in FIELDS4:
            assert np.array_equal(bits(a[s][n]), bits(b[s][n]))


def test_tune_report_lists_every_pair_variant():
    # The report gives each fused-pair stage its chosen variant and every
    # variant's time; the TMA-staged z-march (3) is offered on a level whose
    # x extent is a multiple of 4 (64 and 128 here), and the choice is the
    # fastest of those timed.
    b = Batch(2)
    for c in (Config(NX=128, NY=64, NZ=48, H=1.0 / 128, DT=0.002, Viscosity=1e-4, Density=1.0,
                     Precision=AF_PRECISION_MIXED),
              Config(NX=64, NY=40, NZ=36, H=1.0 / 64, DT=0.002, Viscosity=1e-4, Density=1.0,
                     Precision=AF_PRECISION_MIXED)):
        b.assign(c)
    rep = b.tune(2)
    pairs = {k: v for k, v in rep.items() if "variants_us" in v}
    assert pairs
    for v in pairs.values():
        times = {int(k): t for k, t in v["variants_us"].items() if t >= 0}
        assert {0, 1, 2} <= set(times)
        assert v["variant"] in times and times[v["variant"]] == min(times.values())
    assert any("3" in v["variants_us"] for v in pairs.values())
    b.close()


def test_slots_come_and_go_between_steps():
    b = Batch(4)
    first = [b.assign(c) for c in SHAPES[:3]]
    for s in first:
        for n, a in zip(("U", "V", "W"), seed_fields(b.config(s), s)):
            b.upload(s, n, a)
    b.apply_velocity_bc()
    b.step(2)
    b.release(first[1])
    late = b.assign(SHAPES[4])
    for n, a in zip(("U", "V", "W"), seed_fields(b.config(late), 99)):
        b.upload(late, n, a)
    # Only the new slot needs its BC; applying it to all is idempotent.
    b.apply_velocity_bc()
    b.step(2)
    for s, c, steps, stream in ((first[0], SHAPES[0], 4, first[0]), (first[2], SHAPES[2], 4, first[2]),
                                (late, SHAPES[4], 2, 99)):
        ref = alone(c, stream, steps)
        for n in FIELDS4:
            assert np.array_equal(bits(b.download(s, n)), bits(ref[n])), f"slot {s} field {n}"
    b.close()


def test_inactive_slot_is_left_untouched():
    b = Batch(2)
    s0, s1 = b.assign(SHAPES[0]), b.assign(SHAPES[1])
    for s in (s0, s1):
        for n, a in zip(("U", "V", "W"), seed_fields(b.config(s), s)):
            b.upload(s, n, a)
    b.apply_velocity_bc()
    before = {n: b.download(s1, n).copy() for n in ("U", "V", "W")}
    b.set_active(s1, False)
    b.step(2)
    for n in ("U", "V", "W"):
        assert np.array_equal(bits(b.download(s1, n)), bits(before[n]))
    ref = alone(SHAPES[0], s0, 2)
    assert np.array_equal(bits(b.download(s0, "U")), bits(ref["U"]))
    b.close()


def test_fault_in_one_slot_leaves_the_others_exact():
    b = Batch(3)
    slots = [b.assign(c) for c in SHAPES[:3]]
    for s in slots:
        for n, a in zip(("U", "V", "W"), seed_fields(b.config(s), s)):
            b.upload(s, n, a)
    u = b.download(slots[1], "U")
    f = b.field(slots[1], "U")
    u[5 + 6 * f.SY + 7 * f.SZ] = math.nan
    b.upload(slots[1], "U", u)
    b.apply_velocity_bc()
    b.step(2)
    faulted, msg = b.status(slots[1])
    assert faulted and msg.startswith("aeroflux: guard-page fault contained")
    for s in (slots[0], slots[2]):
        assert not b.status(s)[0]
        ref = alone(SHAPES[s], s, 2)
        assert np.array_equal(bits(b.download(s, "U")), bits(ref["U"]))
    b.close()


def test_pool_admission_refuses_what_does_not_fit():
    c = SHAPES[4]
    need = Batch.slot_bytes(c)
    b = Batch(4, pool_bytes=2 * need + 4096)
    b.assign(c)
    b.assign(c)
    with pytest.raises(AerofluxError):
        b.assign(c)
    b.close()


@pytest.mark.slow
def test_benchmark_batch_reaches_tolerance():
    cfgs = batched_instances(256)
    b = Batch(len(cfgs))
    slots = [b.assign(c) for c in cfgs]
    print(b.tune(3))
    for s in slots:
        for n, a in zip(("U", "V", "W"), seed_fields(b.config(s), s)):
            b.upload(s, n, a)
    b.apply_velocity_bc()
    b.step(2)
    worst = max(b.max_divergence(s) for s in slots)
    print(f"256 uneven grids, 2 steps: worst max|div| {worst:.3e}")
    assert worst <= 1e-10
    # A sample checked against the same grid alone.
    for s in (0, 17, 255):
        ref = alone(cfgs[s], s, 2)
        assert np.array_equal(bits(b.download(s, "U")), bits(ref["U"]))
    # The benchmark configuration's full 300 Steps: every grid stays finite
    # and divergence-free to the tolerance.
    b.step(298)
    worst = max(b.max_divergence(s) for s in slots)
    print(f"256 uneven grids, 300 steps: worst max|div| {worst:.3e}")
    assert worst <= 1e-10
    for s in (3, 101, 200):
        assert np.all(np.isfinite(b.download(s, "U")))
    b.close()


def test_tuning_between_steps_leaves_the_slots_untouched():
    # The server tunes while requests are resident: the autotuner's timing
    # runs of every stage (the gradient included) must leave each slot's
    # state exactly as it was.
    cfgs = SHAPES[:4]
    runs = []
    for tune in (False, True):
        b = Batch(len(cfgs))
        slots = [b.assign(c) for c in cfgs]
        for s in slots:
            for n, a in zip(("U", "V", "W"), seed_fields(b.config(s), s)):
                b.upload(s, n, a)
        b.apply_velocity_bc()
        b.step(2)
        if tune:
            b.tune(2)
        b.step(2)
        runs.append([np.concatenate([bits(b.download(s, n)) for n in FIELDS4]) for s in slots])
        b.close()
    for a, t in zip(*runs):
        assert np.array_equal(a, t)
