"""Parity of the CUDA path (through the C ABI) with the CPU oracle.

The FP64 plain form must reproduce the reference's binary64 arithmetic bit
for bit, so every comparison here is on bit patterns (signed zeros
included), stage by stage and over whole Steps, on shapes that cover cubes,
odd and non-cubic extents, ghost thickness 2, a one-cell-wide grid, CFL far
above 1 (backtraces clamped at the halo) and garbage in every ghost and
never-written plane.  The only tolerance is KineticEnergy's, whose serial
sum the device evaluates as a fixed tree (relative 1e-12).
"""
import math

import numpy as np
import pytest

from aeroflux_gb300 import Config, FaultError, New
from oracle.oracle import OracleEngine, OracleError
from tests.helpers import FID, FIELDS, assert_bit_identical, bits, make_pair, oracle_kwargs

pytestmark = pytest.mark.gpu

SHAPES = {
    "vortex8": (dict(NX=8, NY=8, NZ=8, H=0.125, DT=0.005), "vortex", 1.0),
    "tg12": (dict(NX=12, NY=12, NZ=12, H=1 / 12, DT=0.004, Viscosity=1e-4, GaussSeidelIters=30), "tg", 1.0),
    "odd10x7x5": (dict(NX=10, NY=7, NZ=5, H=0.1, DT=0.003, Viscosity=1e-3, GaussSeidelIters=12), "tg", 1.0),
    "ghost2": (dict(NX=9, NY=6, NZ=11, Ghost=2, H=1 / 11, DT=0.004, Viscosity=5e-4, GaussSeidelIters=10), "tg", 1.0),
    "thin1x3x2": (dict(NX=1, NY=3, NZ=2, H=0.5, DT=0.01, GaussSeidelIters=3), "tg", 1.0),
    "cell1x1x1": (dict(NX=1, NY=1, NZ=1, H=1.0, DT=0.01, GaussSeidelIters=2), "tg", 1.0),
    "line40x1x1": (dict(NX=40, NY=1, NZ=1, H=1 / 40, DT=0.002, Viscosity=1e-3, GaussSeidelIters=5), "tg", 1.0),
    "cfl4": (dict(NX=16, NY=12, NZ=10, H=1 / 16, DT=0.01, Viscosity=1e-5, GaussSeidelIters=6), "tg", 25.0),
    "rect33x17x20": (dict(NX=33, NY=17, NZ=20, H=1 / 33, DT=0.002, Viscosity=1e-5, GaussSeidelIters=8), "tg", 1.0),
}


def _cfg(name):
    kw, kind, amp = SHAPES[name]
    return Config(**kw), kind, amp


def _random_pair(cfg, seed=7):
    """Engines whose every U/V/W element (ghosts and never-written planes
    included) holds random data, so exact write sets are tested too."""
    gpu = New(cfg)
    orc = OracleEngine(**oracle_kwargs(cfg))
    rng = np.random.default_rng(seed)
    for name in ("U", "V", "W"):
        a = rng.normal(size=orc.field(FID[name]).count)
        gpu.upload(name, a)
        orc.data(FID[name])[:] = a
    return gpu, orc


@pytest.mark.parametrize("name", list(SHAPES))
def test_velocity_bc_bit_exact(name):
    cfg, _, _ = _cfg(name)
    gpu, orc = _random_pair(cfg)
    gpu.applyVelocityBC()
    orc.apply_velocity_bc()
    assert_bit_identical(gpu, orc, ["U", "V", "W"], "applyVelocityBC")


@pytest.mark.parametrize("name", list(SHAPES))
@pytest.mark.parametrize("axis", [0, 1, 2])
def test_sweep_bit_exact(name, axis):
    cfg, kind, amp = _cfg(name)
    gpu, orc = make_pair(cfg, kind, amp)
    dt = orc.cfg["dt"] * 0.5
    gpu.applyVelocityBC()
    orc.apply_velocity_bc()
    gpu.sweep(axis, dt)
    orc.sweep(axis, dt)
    assert_bit_identical(gpu, orc, FIELDS, f"sweep axis {axis}")


@pytest.mark.parametrize("name", ["tg12", "odd10x7x5", "ghost2", "thin1x3x2"])
def test_sweep_bit_exact_with_garbage_halo(name):
    cfg, _, _ = _cfg(name)
    gpu, orc = _random_pair(cfg, seed=11)
    dt = orc.cfg["dt"] * 0.5
    for axis in (0, 1, 2):
        gpu.applyVelocityBC()
        orc.apply_velocity_bc()
        gpu.sweep(axis, dt)
        orc.sweep(axis, dt)
    assert_bit_identical(gpu, orc, FIELDS, "three sweeps")


EXTREMES = {
    # 2^1023 = 8.98846567e307: the shortcut's threshold lies between the two.
    "finite": [0.0, -0.0, 1.7e308, -1.7e308, 8.98e307, -8.98e307, 8.99e307, -8.99e307, 5e-324, -5e-324],
    "inf": [0.0, -0.0, 1.7e308, -1.7e308, math.inf, -math.inf, 5e-324],
}


@pytest.mark.parametrize("name", ["tg12", "odd10x7x5", "rect33x17x20"])
@pytest.mark.parametrize("seed", [1, 2, 3])
@pytest.mark.parametrize("kind", list(EXTREMES))
def test_sweep_bit_exact_with_extreme_values(name, seed, kind):
    # Signed zeros, magnitudes near the top of binary64 (zero-weight lerps
    # of them overflow), infinities (clamped backtraces, Inf * 0 = NaN) and
    # subnormals, planted among ordinary values in every field: the sweeps'
    # shortcuts for zero-weight lerps must reproduce the reference in all of
    # these cases.  A face velocity that averages +Inf with -Inf is NaN, a
    # contained fault: then both must report the same fault (single-worker
    # oracle order) and hold the same U, V, W.
    cfg, _, _ = _cfg(name)
    gpu = New(cfg)
    kw = oracle_kwargs(cfg)
    kw["workers"] = 1
    orc = OracleEngine(**kw)
    rng = np.random.default_rng(100 + seed)
    specials = np.array(EXTREMES[kind])
    for name_f in ("U", "V", "W"):
        a = rng.normal(size=orc.field(FID[name_f]).count)
        pick = rng.random(a.size) < 0.03
        a[pick] = rng.choice(specials, size=int(pick.sum()))
        zeros = rng.random(a.size) < 0.04
        a[zeros] = rng.choice([0.0, -0.0], size=int(zeros.sum()))
        orc.data(FID[name_f])[:] = a
        gpu.upload(name_f, a)
    dt = orc.cfg["dt"] * 0.5
    for axis in (0, 1, 2):
        ofault = gfault = None
        try:
            orc.sweep(axis, dt)
        except OracleError as ex:
            ofault = str(ex)
        try:
            gpu.sweep(axis, dt)
        except FaultError as ex:
            gfault = str(ex)
        assert gfault == ofault
        if ofault:
            assert_bit_identical(gpu, orc, ["U", "V", "W"], f"state after the fault in sweep axis {axis}")
            break
        assert_bit_identical(gpu, orc, ["U", "V", "W", "Tmp0", "Tmp1", "Tmp2"], f"sweep axis {axis}")
    orc.close()


@pytest.mark.parametrize("name", list(SHAPES))
def test_projection_stages_bit_exact(name):
    cfg, kind, amp = _cfg(name)
    gpu, orc = make_pair(cfg, kind, amp)
    gpu.computeDivergence()
    orc.compute_divergence()
    assert_bit_identical(gpu, orc, ["Div"], "computeDivergence")
    gpu.solvePressureRedBlack()
    orc.solve_pressure_red_black()
    assert_bit_identical(gpu, orc, ["P"], "solvePressureRedBlack")
    gpu.subtractGradient()
    orc.subtract_gradient()
    assert_bit_identical(gpu, orc, ["U", "V", "W"], "subtractGradient")


@pytest.mark.parametrize("name", list(SHAPES))
def test_pressure_bc_bit_exact(name):
    cfg, _, _ = _cfg(name)
    gpu = New(cfg)
    orc = OracleEngine(**oracle_kwargs(cfg))
    a = np.random.default_rng(3).normal(size=orc.field(0).count)
    gpu.upload("P", a)
    orc.data(0)[:] = a
    gpu.applyPressureBC()
    orc.apply_pressure_bc()
    assert_bit_identical(gpu, orc, ["P"], "applyPressureBC")


@pytest.mark.parametrize("name", list(SHAPES))
def test_project_bit_exact(name):
    cfg, kind, amp = _cfg(name)
    gpu, orc = make_pair(cfg, kind, amp)
    gpu.project()
    orc.project()
    assert_bit_identical(gpu, orc, FIELDS, "project")


@pytest.mark.parametrize("name,steps", [("vortex8", 3), ("tg12", 5), ("odd10x7x5", 4), ("ghost2", 3),
                                        ("thin1x3x2", 4), ("cfl4", 2), ("rect33x17x20", 3)])
def test_step_bit_exact(name, steps):
    cfg, kind, amp = _cfg(name)
    gpu, orc = make_pair(cfg, kind, amp)
    gpu.Step(steps)
    orc.step(steps)
    assert_bit_identical(gpu, orc, FIELDS, f"{steps} steps")
    assert gpu.MaxDivergence() == orc.max_divergence()
    assert gpu.MaxVelocity() == orc.max_velocity()
    assert gpu.CFL() == orc.cfl()
    ke_g, ke_o = gpu.KineticEnergy(), orc.kinetic_energy()
    assert abs(ke_g - ke_o) <= 1e-12 * abs(ke_o)


def test_step_with_garbage_halo_bit_exact():
    cfg, _, _ = _cfg("odd10x7x5")
    gpu, orc = _random_pair(cfg, seed=5)
    gpu.Step(2)
    orc.step(2)
    assert_bit_identical(gpu, orc, FIELDS, "2 steps from random halo")


def test_shear_layer_example_bit_exact():
    # example_test.go:13-61 with the README's 60-sweep row (README.md:366-377).
    cfg = Config(NX=16, NY=16, NZ=16, H=1 / 16, DT=0.004, Viscosity=1e-5, Density=1.0, GaussSeidelIters=60)
    gpu, orc = make_pair(cfg, "shear")
    gpu.Step(10)
    orc.step(10)
    assert_bit_identical(gpu, orc, FIELDS, "shear layer")
    assert f"{gpu.MaxDivergence():.1e}" == "5.1e-03"


def test_results_identical_run_to_run():
    cfg, kind, amp = _cfg("tg12")
    outs = []
    for _ in range(2):
        gpu, _ = make_pair(cfg, kind, amp)
        gpu.Step(3)
        outs.append(np.concatenate([bits(gpu.download(n)) for n in FIELDS]))
        gpu.Close()
    assert np.array_equal(outs[0], outs[1])


def test_mesh_data_views_alias_like_the_reference():
    # Callers seed through Mesh.Data views and read results back through them.
    cfg = Config(NX=8, NY=8, NZ=8, H=0.125, DT=0.005)
    e = New(cfg)
    orc = OracleEngine(**oracle_kwargs(cfg))
    orc.seed_vortex(1.0)
    m = e.Mesh
    u = m.Data(m.U)
    u[:] = orc.data(1)
    m.Data(m.V)[:] = orc.data(2)
    m.Data(m.W)[:] = orc.data(3)
    e.Step()
    orc.step()
    assert np.array_equal(bits(u), bits(orc.data(1)))
    e.Close()
    e.Close()  # idempotent


# --- contained faults --------------------------------------------------------

@pytest.mark.parametrize("field,cell", [("U", (4, 4, 4)), ("V", (3, 5, 2)), ("W", (6, 2, 5)), ("U", (2, 1, 1))])
def test_nan_fault_message_and_state_match_oracle(field, cell):
    cfg = Config(NX=8, NY=8, NZ=8, H=0.125, DT=0.005)
    gpu, orc = make_pair(cfg, "vortex", 1.0, oracle_workers=1)
    f = orc.field(FID[field])
    x, y, z = cell
    idx = x + y * f.sy + z * f.sz
    a = gpu.download(field)
    a[idx] = math.nan
    gpu.upload(field, a)
    orc.data(FID[field])[idx] = math.nan
    with pytest.raises(OracleError) as oex:
        orc.step()
    with pytest.raises(FaultError) as gex:
        gpu.Step()
    assert str(gex.value) == str(oex.value)
    assert str(gex.value).startswith("aeroflux: guard-page fault contained: runtime error: index out of range [")
    # Both stop before the faulting sweep's commit: the current U, V, W and P
    # descriptors hold identical data (the faulting sweep only wrote Tmp).
    assert_bit_identical(gpu, orc, ["U", "V", "W", "P", "Div"], "state after fault")


def test_fault_stops_multi_step_call_and_engine_stays_usable():
    cfg = Config(NX=8, NY=8, NZ=8, H=0.125, DT=0.005)
    gpu, orc = make_pair(cfg, "vortex", 1.0, oracle_workers=1)
    gpu.Step(2)
    orc.step(2)
    u = gpu.download("U")
    u[5 + 3 * 11 + 4 * 11 * 10] = math.nan
    gpu.upload("U", u)
    orc.data(1)[5 + 3 * 11 + 4 * 11 * 10] = math.nan
    with pytest.raises(FaultError):
        gpu.Step(5)
    with pytest.raises(OracleError):
        orc.step()
    assert_bit_identical(gpu, orc, ["U", "V", "W"], "state after fault in a 5-step call")
    # A fresh field makes the engine usable again.
    fresh, _ = make_pair(cfg, "vortex", 1.0)
    for n in ("U", "V", "W"):
        gpu.upload(n, fresh.download(n))
    gpu.Step(1)
    assert math.isfinite(gpu.MaxDivergence())


def test_inf_velocity_is_clamped_not_faulted():
    # stencil.go:174-188 clamps +-Inf coordinates into the halo: no fault.
    cfg = Config(NX=8, NY=8, NZ=8, H=0.125, DT=0.005)
    gpu, orc = make_pair(cfg, "vortex", 1.0, oracle_workers=1)
    u = gpu.download("U")
    u[4 + 4 * 11 + 4 * 11 * 10] = math.inf
    gpu.upload("U", u)
    orc.data(1)[4 + 4 * 11 + 4 * 11 * 10] = math.inf
    gpu.applyVelocityBC()
    orc.apply_velocity_bc()
    gpu.sweep(0, 0.0025)
    orc.sweep(0, 0.0025)
    assert_bit_identical(gpu, orc, FIELDS, "x sweep with an Inf velocity")


def test_enable_sparse_solver_reports_reference_text():
    e = New(Config(NX=4, NY=4, NZ=4))
    with pytest.raises(Exception) as ex:
        e.EnableSparseSolver()
    assert "sparse direct solver requires darwin with cgo" in str(ex.value)
