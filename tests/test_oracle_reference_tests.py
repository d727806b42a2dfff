"""The reference's engine tests (AeroFlex/engine_test.go, example_test.go),
restated against the CPU oracle.  They pin the oracle to every property the
reference asserts for this path, the way the reference pins itself."""
import math

import numpy as np
import pytest

from oracle.oracle import OracleEngine, OracleError, P, U, V, W, mac_bytes, normalize


def test_config_normalize_defaults():  # engine_test.go:18-35
    c, err = normalize(nx=16, ny=16, nz=16)
    assert err is None
    assert c["ghost"] == 1 and c["density"] == 1
    assert c["h"] > 0 and c["dt"] > 0 and c["workers"] >= 1
    assert c["gauss_seidel_iters"] == 24


@pytest.mark.parametrize("kw", [
    dict(nx=0, ny=8, nz=8), dict(nx=-4, ny=8, nz=8), dict(nx=8, ny=8, nz=8, ghost=-1),
    dict(nx=8, ny=8, nz=8, viscosity=-1), dict(nx=8, ny=8, nz=8, h=math.nan),
    dict(nx=8, ny=8, nz=8, dt=math.inf), dict(nx=8, ny=8, nz=8, density=-2),
    dict(nx=8, ny=8, nz=8, h=0.1, viscosity=1.0, dt=1.0)])
def test_config_normalize_rejects(kw):  # engine_test.go:37-59
    _, err = normalize(**kw)
    assert err is not None and err.startswith("aeroflux: ")


def test_config_workers_capped_by_depth():  # engine_test.go:61-69
    c, err = normalize(nx=8, ny=8, nz=2, workers=64)
    assert err is None and c["workers"] <= 2


def test_mac_staggered_extents_and_strides():  # engine_test.go:71-90, arena_test.go:215-237
    with OracleEngine(nx=8, ny=6, nz=4) as e:
        p, u, v, w = (e.field(i) for i in (P, U, V, W))
        assert (u.nx, u.ny, u.nz) == (p.nx + 1, p.ny, p.nz)
        assert (v.nx, v.ny, v.nz) == (p.nx, p.ny + 1, p.nz)
        assert (w.nx, w.ny, w.nz) == (p.nx, p.ny, p.nz + 1)
    with OracleEngine(nx=64, ny=32, nz=16) as e:
        p = e.field(P)
        assert (p.sy, p.sz) == (66, 66 * 34)
        offs = [e.field(i).off for i in range(8)]
        assert all(o % 128 == 0 for o in offs) and offs == sorted(offs)
        assert mac_bytes(64, 32, 16, 1) > offs[-1]


def test_projection_removes_divergence():  # engine_test.go:108-130
    with OracleEngine(nx=16, ny=16, nz=16, h=1 / 16, dt=0.01, density=1.0, gauss_seidel_iters=200) as e:
        e.seed_vortex(1.0)
        before = e.max_divergence()
        assert before > 0
        e.project()
        assert e.max_divergence() <= before / 50


def _run(workers, steps=5):
    with OracleEngine(nx=12, ny=12, nz=12, h=1 / 12, dt=0.005, density=1.0, viscosity=0.0,
                      workers=workers, gauss_seidel_iters=30) as e:
        e.seed_vortex(1.0)
        e.step(steps)
        return np.concatenate([e.data(U).copy(), e.data(V).copy(), e.data(W).copy()])


def test_step_is_deterministic_across_worker_counts():  # engine_test.go:134-170
    ref = _run(1)
    for w in (2, 3, 4, 8):
        assert np.array_equal(ref.view(np.uint64), _run(w).view(np.uint64)), f"workers={w}"


def test_step_is_reproducible_across_runs():  # engine_test.go:174-193
    def ke():
        with OracleEngine(nx=10, ny=10, nz=10, h=0.1, dt=0.004, workers=4, gauss_seidel_iters=20) as e:
            e.seed_vortex(1.0)
            e.step(8)
            return e.kinetic_energy()
    assert ke() == ke()


def test_step_stays_finite():  # engine_test.go:195-218
    with OracleEngine(nx=12, ny=12, nz=12, h=1 / 12, dt=0.01, viscosity=1e-4, gauss_seidel_iters=25) as e:
        e.seed_vortex(2.0)
        e.step(30)
        for f in (U, V, W, P):
            assert np.all(np.isfinite(e.data(f)))


def test_step_leaves_field_divergence_free():  # engine_test.go:225-243
    with OracleEngine(nx=12, ny=12, nz=12, h=1 / 12, dt=0.005, gauss_seidel_iters=300) as e:
        e.seed_vortex(1.0)
        for _ in range(5):
            e.step()
            assert e.max_divergence() <= 1e-3


def test_no_slip_walls_hold_normal_velocity():  # engine_test.go:247-268
    with OracleEngine(nx=8, ny=8, nz=8, h=0.125, dt=0.005) as e:
        e.seed_vortex(1.0)
        e.step(3)
        u = e.view3(U)
        assert np.all(u[1:9, 1:9, 1] == 0) and np.all(u[1:9, 1:9, 9] == 0)


def test_example_shear_layer():  # example_test.go:13-61
    with OracleEngine(nx=16, ny=16, nz=16, h=1 / 16, dt=0.004, viscosity=1e-5, density=1.0,
                      gauss_seidel_iters=400) as e:
        e.seed_shear_layer()
        e.step(10)
        assert not math.isnan(e.kinetic_energy())
        assert e.max_divergence() < 1e-3


def test_nan_backtrace_is_a_contained_fault():
    # arena.go:230-243 + aeroflux.go:286-324: on amd64 a NaN coordinate
    # becomes INT64_MIN and Go's bounds check panics; Step returns the text.
    with OracleEngine(nx=8, ny=8, nz=8, h=0.125, dt=0.005, workers=1) as e:
        e.seed_vortex(1.0)
        e.view3(U)[4, 4, 4] = math.nan
        with pytest.raises(OracleError) as ex:
            e.step()
        msg = str(ex.value)
        assert msg.startswith("aeroflux: guard-page fault contained: runtime error: index out of range [")


def test_nan_where_go_does_not_fault_propagates():
    # With even padded row strides the wrapped INT64_MIN*SY vanishes mod 2^64
    # and Go reads in-range taps: no fault, NaN flows on.  A lone NaN in V at
    # a 8^3 grid faults only in the y sweep, through component U.
    with OracleEngine(nx=8, ny=8, nz=8, h=0.125, dt=0.005, workers=1) as e:
        e.seed_vortex(1.0)
        e.view3(V)[4, 4, 4] = math.nan
        e.apply_velocity_bc()
        e.sweep(0, 0.0025)  # x sweep: no fault
        assert np.isnan(e.view3(V)).any()
        with pytest.raises(OracleError):
            e.sweep(1, 0.0025)


def test_close_is_idempotent():  # engine_test.go:290-298
    e = OracleEngine(nx=8, ny=8, nz=8)
    e.close()
    e.close()
