"""The oracle's MacCormack advection (the restatement the GPU's MacCormack
sweeps are compared with bit for bit): on the CPU it must translate a sine
wave with at most half the reference semi-Lagrangian sweep's error, leave a
uniform field exactly uniform, and switching back must give the reference
sweep's bits again."""
import math

import numpy as np

from oracle.oracle import OracleEngine

U, V, W = 1, 2, 3
MACCORMACK, SEMI_LAGRANGIAN = 1, 0


def translate_error(scheme, sweeps=20, u0=0.5, cells_per_wave=16):
    nx, ny, nz = 64, 6, 6
    h = 1.0 / nx
    dt = 0.3 * h / u0  # 0.3 cells per sweep
    with OracleEngine(nx=nx, ny=ny, nz=nz, h=h, dt=dt, viscosity=0.0, workers=1) as o:
        o.set_advection(scheme)
        fv = o.field(V)
        gx = np.arange(fv.nx)

        def profile(shift):
            row = np.sin(2 * math.pi * (gx - 1 + 0.5 - shift) / cells_per_wave)
            return np.broadcast_to(row, (fv.nz, fv.ny, fv.nx)).ravel().copy()

        v = profile(0.0)
        for _ in range(sweeps):
            o.data(U)[:] = u0
            o.data(V)[:] = v
            o.data(W)[:] = 0.0
            o.sweep(0, dt)
            v = o.data(V).copy()
        exact = profile(sweeps * 0.3)
    sel = np.zeros((fv.nz, fv.ny, fv.nx), bool)
    sel[1:-1, 1:-1, 16:48] = True
    d = v.reshape(sel.shape)[sel] - exact.reshape(sel.shape)[sel]
    return float(np.max(np.abs(d)))


def test_maccormack_translates_a_wave_more_accurately():
    assert translate_error(MACCORMACK) < 0.5 * translate_error(SEMI_LAGRANGIAN)


def test_uniform_field_stays_uniform():
    # Without viscosity, faces a few cells from the (zeroed) walls see only
    # the uniform value: the forward step, the backward trace and the
    # correction all return it exactly.
    with OracleEngine(nx=12, ny=10, nz=9, h=1 / 12, dt=0.004, viscosity=0.0, workers=2) as o:
        o.set_advection(MACCORMACK)
        for f in (U, V, W):
            o.data(f)[:] = 0.25
        o.apply_velocity_bc()
        for axis in range(3):
            o.sweep(axis, 0.002)
        for f in (U, V, W):
            d = o.field(f)
            a = o.data(f).reshape(d.nz, d.ny, d.nx)
            assert np.all(a[3:-3, 3:-3, 3:-3] == 0.25)


def test_switching_back_gives_the_reference_bits():
    def run(switch):
        with OracleEngine(nx=12, ny=10, nz=9, h=1 / 12, dt=0.004, viscosity=1e-5, workers=2) as o:
            o.seed_taylor_green(1.0, 0.01, 42, 0)
            o.apply_velocity_bc()
            if switch:
                o.set_advection(MACCORMACK)
                o.set_advection(SEMI_LAGRANGIAN)
            o.step(2)
            return [o.data(f).copy() for f in (U, V, W, 0)]
    for a, b in zip(run(False), run(True)):
        assert np.array_equal(a.view(np.uint64), b.view(np.uint64))


def test_same_bits_for_any_worker_count():
    # The forward step and the correction run over the same z shards as the
    # reference sweep; the result does not depend on how many there are.
    def run(workers):
        with OracleEngine(nx=12, ny=12, nz=12, h=1 / 12, dt=0.004, viscosity=1e-5, workers=workers) as o:
            o.seed_taylor_green(1.0, 0.01, 42, 0)
            o.apply_velocity_bc()
            o.set_advection(MACCORMACK)
            o.step(2)
            return np.concatenate([o.data(f).copy() for f in (U, V, W, 0)])
    ref = run(1)
    for w in (2, 3, 4, 8):
        assert np.array_equal(ref.view(np.uint64), run(w).view(np.uint64)), f"workers={w}"
