"""Bit-level parity of the mixed-precision, batched and served forms with the
binary32 restatement of their arithmetic (oracle/mixed_oracle.c).

The mixed form trades the reference's bits for speed, but it is itself
deterministic: every binary32 and binary64 operation has an explicit rounding
and a fixed evaluation order.  So the CUDA kernels must reproduce the
restatement bit for bit: one binary32 sweep per axis, one V-cycle, whole
refinement solves with the adaptive V-cycle control, and whole Steps, on
cubes, odd and non-cubic extents, the fused pair's wide and narrow tile
columns (nx = 32, 96, 33, 65, 97), degenerate axes, grids whose coarsest
level is too large for the one-block tail, odd smoothing counts, and slots of
uneven batches.  The last tests plant mistakes into the restatement and show
that these comparisons catch them.
"""
import contextlib
import os

import numpy as np
import pytest

from aeroflux_gb300 import AF_PRECISION_MIXED, Config, New
from aeroflux_gb300.batch import Batch
from aeroflux_gb300.workloads import batched_instances, taylor_green
from oracle import oracle as fp64_oracle
from oracle import mixed as mixed_oracle
from oracle.mixed import MixedOracle
from tests.helpers import FIELDS, make_pair, same_bits

pytestmark = pytest.mark.gpu

SHAPES = [(16, 16, 16), (32, 32, 32), (96, 40, 36), (33, 17, 20), (65, 24, 16), (97, 34, 18), (24, 20, 18),
          (48, 32, 96), (1, 1, 1), (40, 1, 1), (3, 2, 5), (35, 33, 37)]
ENV_KEYS = ("AEROFLUX_FIXED_REFINEMENT_PASSES", "AEROFLUX_MG_VCYCLES", "AEROFLUX_COLD_START",
            "AEROFLUX_MG_PER_LEVEL", "AEROFLUX_MG_PAIRS", "AEROFLUX_MG_PASS_FLOOR", "AEROFLUX_SWEEP_ROWS",
            "AEROFLUX_PAIR_VARIANT")
# The staged tile sweep (default) and the row sweep compute the same bits.
SWEEPS = {"staged": {}, "rows": {"AEROFLUX_SWEEP_ROWS": 1}}


@contextlib.contextmanager
def env(**kw):
    old = {k: os.environ.get(k) for k in ENV_KEYS}
    for k in ENV_KEYS:
        os.environ.pop(k, None)
    os.environ.update({k: str(v) for k, v in kw.items()})
    try:
        yield
    finally:
        for k, v in old.items():
            if v is None:
                os.environ.pop(k, None)
            else:
                os.environ[k] = v


def mixed_cfg(n, **kw):
    nx, ny, nz = n
    base = dict(NX=nx, NY=ny, NZ=nz, H=1.0 / max(n), DT=0.004, Viscosity=1e-4, Density=1.0,
                Precision=AF_PRECISION_MIXED, DivTol=1e-10)
    base.update(kw)
    return Config(**base)


def oracle_for(cfg: Config, **kw) -> MixedOracle:
    c = Config(**{k: getattr(cfg, k) for k, _ in Config._MAP})
    c.Normalize()
    return MixedOracle(c.NX, c.NY, c.NZ, c.H, c.DT, c.Viscosity, c.Density, c.Ghost, c.DivTol, c.InnerSweeps,
                       c.MaxRefine, **kw)


def make_mixed_pair(n, amp=1.0, noise=0.01, apply_bc=True, env_kw=None, orc_kw=None, **cfg_kw):
    cfg = mixed_cfg(n, **cfg_kw)
    with env(**(env_kw or {})):
        e = New(cfg)
    o = oracle_for(e.Cfg, **(orc_kw or {}))
    u, v, w = taylor_green(e.Cfg, amp, noise)
    for i, (name, a) in enumerate((("U", u), ("V", v), ("W", w)), start=1):
        e.upload(name, a)
        o.data(i)[:] = a
    if apply_bc:
        e.applyVelocityBC()
        o.apply_velocity_bc()
    return e, o


def assert_same(gpu_fields, orc, names=FIELDS, what=""):
    for i, name in enumerate(FIELDS):
        if name not in names:
            continue
        g = gpu_fields(name)
        ref = orc.data(i)
        ok = same_bits(g, ref)
        if not ok.all():
            bad = np.nonzero(~ok)[0]
            raise AssertionError(f"{what} {name}: {bad.size} of {g.size} differ; first at {bad[0]}: "
                                 f"gpu={g[bad[0]]!r} oracle={ref[bad[0]]!r}")


@pytest.mark.parametrize("kind", sorted(SWEEPS))
@pytest.mark.parametrize("n", SHAPES)
@pytest.mark.parametrize("axis", [0, 1, 2])
def test_binary32_sweep_bit_exact(n, axis, kind):
    e, o = make_mixed_pair(n, env_kw=SWEEPS[kind])
    e.sweep(axis, 0.002)
    o.sweep(axis, 0.002)
    assert_same(e.download, o, ("U", "V", "W", "Tmp0", "Tmp1", "Tmp2"), f"{n} axis {axis}")
    e.Close()


@pytest.mark.parametrize("kind", sorted(SWEEPS))
@pytest.mark.parametrize("axis", [0, 1, 2])
def test_binary32_sweep_random_ghosts_and_clamped_backtraces(axis, kind):
    # Random data in every element (ghosts and never-written planes
    # included, no BC) at amplitude 25: backtraces leave the field and clamp,
    # most of them beyond the staged halo (the global fallback).
    n = (20, 14, 11)
    e, o = make_mixed_pair(n, apply_bc=False, env_kw=SWEEPS[kind])
    rng = np.random.default_rng(7 + axis)
    for i, name in enumerate(("U", "V", "W"), start=1):
        a = rng.uniform(-25, 25, o.data(i).size)
        e.upload(name, a)
        o.data(i)[:] = a
    e.sweep(axis, 0.01)
    o.sweep(axis, 0.01)
    assert_same(e.download, o, ("U", "V", "W", "Tmp0", "Tmp1", "Tmp2"), f"random ghosts axis {axis}")
    e.Close()


@pytest.mark.parametrize("n", SHAPES)
def test_one_vcycle_bit_exact(n):
    # One refinement pass of one V-cycle: residual, smoothing, restriction,
    # the tail or the large-coarsest smoothing, prolongation, correction.
    e, o = make_mixed_pair(n, env_kw={"AEROFLUX_FIXED_REFINEMENT_PASSES": 1, "AEROFLUX_MG_VCYCLES": 1},
                           orc_kw={"fixed_passes": 1, "vcycles": 1})
    e.project()
    o.project()
    assert_same(e.download, o, ("P", "U", "V", "W", "Div"), f"{n} one V-cycle")
    e.Close()


@pytest.mark.parametrize("n", SHAPES)
def test_refined_projection_bit_exact(n):
    e, o = make_mixed_pair(n)
    e.project()
    o.project()
    passes, _ = e.LastProjectionStats()
    assert passes == o.passes and e.LastProjectionVCycles() == o.vcycles
    assert_same(e.download, o, ("P", "U", "V", "W", "Div"), f"{n} projection")
    e.Close()


@pytest.mark.parametrize("n", [(16, 16, 16), (33, 17, 20), (96, 40, 36), (65, 24, 16), (1, 1, 1), (40, 1, 1),
                               (35, 33, 37)])
def test_steps_bit_exact(n):
    # Whole Steps: the V-cycle count of later projections follows the
    # reduction factor earlier ones measured (kept across projections), and
    # each projection starts from the last pressure.
    e, o = make_mixed_pair(n)
    for k in range(3):
        e.Step(1)
        o.step(1)
        passes, _ = e.LastProjectionStats()
        assert passes == o.passes, f"step {k}"
        assert_same(e.download, o, FIELDS, f"{n} step {k}")
    e.Close()


@pytest.mark.parametrize("sweeps", [1, 3])
def test_odd_smoothing_counts_bit_exact(sweeps):
    # Odd counts smooth with in-place colour sweeps instead of fused pairs.
    e, o = make_mixed_pair((48, 32, 40), InnerSweeps=sweeps)
    e.Step(2)
    o.step(2)
    assert_same(e.download, o, FIELDS, f"inner sweeps {sweeps}")
    e.Close()


def test_cold_start_fixed_passes_bit_exact():
    e, o = make_mixed_pair((32, 24, 40), env_kw={"AEROFLUX_COLD_START": 1, "AEROFLUX_FIXED_REFINEMENT_PASSES": 2},
                           orc_kw={"warm": False, "fixed_passes": 2})
    e.Step(2)
    o.step(2)
    assert_same(e.download, o, FIELDS, "cold start, two fixed passes")
    e.Close()


def test_per_level_kernels_bit_exact():
    e, o = make_mixed_pair((64, 48, 32), env_kw={"AEROFLUX_MG_PER_LEVEL": 1, "AEROFLUX_MG_PAIRS": 0})
    e.Step(2)
    o.step(2)
    assert_same(e.download, o, FIELDS, "per-level kernels")
    e.Close()


@pytest.mark.parametrize("var", [0, 1, 2, 3, 4])
@pytest.mark.parametrize("n", [(96, 40, 36), (48, 32, 96), (36, 33, 37), (65, 24, 16), (128, 20, 12),
                               (196, 20, 18)])
def test_pair_tile_variants_bit_exact(n, var):
    # Every tile variant of the fused pair, the TMA-staged z-march (3)
    # included, computes the same bits: z chunks of 16 planes with ragged
    # last chunks (nz = 36, 37, 18), ragged y tiles (ny = 33, 20), columns
    # past the x extent (nx = 36, 48) and columns clear of both x walls
    # (nx = 196).  Variant 3 runs on levels whose x extent is a multiple of
    # 4 and variant 1 on the others (nx = 65, 33, ...).
    e, o = make_mixed_pair(n, env_kw={"AEROFLUX_PAIR_VARIANT": var})
    for k in range(2):
        e.Step(1)
        o.step(1)
        assert e.LastProjectionStats()[0] == o.passes, f"step {k}"
        assert_same(e.download, o, FIELDS, f"{n} pair variant {var} step {k}")
    e.Close()


def test_staged_pair_falls_back_for_a_later_slot():
    # A slot assigned after its levels chose the staged pair but without the
    # pair's tensor maps (nx = 66 is not a multiple of 4) switches those
    # levels back to plain tiles; both slots keep the restatement's bits.
    with env(AEROFLUX_PAIR_VARIANT=3):
        b = Batch(2)
    orcs = {}

    def add(cfg, k):
        s = b.assign(cfg)
        o = oracle_for(b.config(s))
        u, v, w = taylor_green(b.config(s), 1.0, 0.01, 42, k)
        for i, (name, a) in enumerate((("U", u), ("V", v), ("W", w)), start=1):
            b.upload(s, name, a)
            o.data(i)[:] = a
        o.apply_velocity_bc()
        orcs[s] = o
        return s

    s0 = add(mixed_cfg((64, 32, 24)), 0)
    b.apply_velocity_bc()
    b.step(1)
    orcs[s0].step(1)
    s1 = add(mixed_cfg((66, 20, 16)), 1)
    b.set_active(s0, False)
    b.apply_velocity_bc()
    b.set_active(s0, True)
    b.step(2)
    for s, o in orcs.items():
        o.step(2)
        assert_same(lambda name: b.download(s, name), o, FIELDS, f"slot {s}")
    b.close()


@pytest.mark.parametrize("pair_var", [None, 3])
def test_batched_slots_bit_exact(pair_var):
    # Uneven slots of the batched workload's generator (the smaller ones,
    # so the oracle stays quick) plus odd extents, stepping in one batch
    # (with the size-chosen pair tiles, and with the staged pair forced).
    cfgs = [c for c in batched_instances(64) if c.NX * c.NY * c.NZ <= 64 * 64 * 48][:6]
    cfgs += [mixed_cfg((33, 17, 20)), mixed_cfg((65, 24, 16), Viscosity=3e-5)]
    with env(**({} if pair_var is None else {"AEROFLUX_PAIR_VARIANT": pair_var})):
        b = Batch(len(cfgs))
    orcs, slots = [], []
    for k, c in enumerate(cfgs):
        s = b.assign(c)
        o = oracle_for(b.config(s))
        u, v, w = taylor_green(b.config(s), 1.0, 0.01, 42, k)
        for i, (name, a) in enumerate((("U", u), ("V", v), ("W", w)), start=1):
            b.upload(s, name, a)
            o.data(i)[:] = a
        o.apply_velocity_bc()
        slots.append(s)
        orcs.append(o)
    b.apply_velocity_bc()
    b.step(3)
    for o in orcs:
        o.step(3)
    for s, o in zip(slots, orcs):
        assert_same(lambda name: b.download(s, name), o, FIELDS, f"slot {s}")
        assert b.projection_stats(s)[0] == o.passes
    b.close()


def test_device_seeded_slot_bit_exact():
    # The served form seeds requests on the device; from that field, a slot
    # steps exactly as the restatement does.
    c = mixed_cfg((48, 40, 32), DT=0.002)
    b = Batch(1)
    s = b.assign(c)
    b.seed(s, 1.0, 0.01, 42, 5)
    o = oracle_for(b.config(s))
    for i, name in enumerate(("U", "V", "W"), start=1):
        o.data(i)[:] = b.download(s, name)
    b.apply_velocity_bc()
    o.apply_velocity_bc()
    b.step(2)
    o.step(2)
    assert_same(lambda name: b.download(s, name), o, FIELDS, "device-seeded slot")
    b.close()


# --- the comparisons catch planted mistakes ---------------------------------

@pytest.mark.parametrize("mutation,n", [(1, (24, 20, 18)), (2, (24, 20, 18)), (3, (24, 20, 18)), (4, (40, 1, 1))])
def test_mutated_mixed_oracle_is_caught(mutation, n):
    # The mutation is in force while the restatement plans its hierarchy
    # (mutation 4 acts there) and while it steps.
    mixed_oracle.set_mutation(mutation)
    try:
        e, o = make_mixed_pair(n)
        e.Step(1)
        o.step(1)
    finally:
        mixed_oracle.set_mutation(0)
    with pytest.raises(AssertionError):
        assert_same(e.download, o, FIELDS, f"mutation {mutation}")
    e.Close()


@pytest.mark.parametrize("mutation", [1, 2, 3, 4, 5])
def test_mutated_fp64_oracle_is_caught(mutation):
    # Random data in the ghosts before the first BC, so the reflection
    # order decides edge values; two Steps of the FP64 form.
    from tests.helpers import assert_bit_identical
    cfg = Config(NX=14, NY=12, NZ=10, H=1 / 14, DT=0.004, Viscosity=1e-4, GaussSeidelIters=6)
    gpu, orc = make_pair(cfg, "tg", 1.0, 0.01, apply_bc=False)
    rng = np.random.default_rng(3)
    for i, name in enumerate(("U", "V", "W"), start=1):
        a = orc.data(i).copy()
        ghost = a == 0.0
        a[ghost] = rng.uniform(-1, 1, int(ghost.sum()))
        gpu.upload(name, a)
        orc.data(i)[:] = a
    gpu.applyVelocityBC()
    gpu.Step(2)
    fp64_oracle.set_mutation(mutation)
    try:
        orc.apply_velocity_bc()
        orc.step(2)
    finally:
        fp64_oracle.set_mutation(0)
    with pytest.raises(AssertionError):
        assert_bit_identical(gpu, orc, FIELDS, f"mutation {mutation}")
    gpu.Close()
    orc.close()
