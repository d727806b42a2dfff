"""MacCormack advection in the FP64 form: the higher-order scheme the
reference names as the remedy for semi-Lagrangian dissipation (README "Known
limitations"; Selle et al. 2008).

Its sweeps and whole Steps equal the oracle's restatement bit for bit.
Against the exact translation of a sine wave it must at least halve the
reference semi-Lagrangian sweep's error, a Taylor-Green vortex must lose
less kinetic energy over the same Steps, and switching back must restore
bit-exact parity with the reference sweep.
"""
import math

import numpy as np
import pytest

from aeroflux_gb300 import (AF_ADVECTION_MACCORMACK, AF_ADVECTION_SEMI_LAGRANGIAN, AF_PRECISION_MIXED,
                            AerofluxError, Config, New)
from aeroflux_gb300.engine import FaultError
from oracle.oracle import OracleError
from tests.helpers import FID, assert_bit_identical, make_pair

pytestmark = pytest.mark.gpu


def translate_error(scheme, sweeps=20, u0=0.5, cells_per_wave=16):
    """Advects V = sin(2 pi x / L) along x in a uniform U through the sweep
    hook and returns the max and RMS of V - exact over the interior away
    from the ends."""
    nx, ny, nz = 64, 6, 6
    h = 1.0 / nx
    dt = 0.3 * h / u0  # 0.3 cells per sweep
    e = New(Config(NX=nx, NY=ny, NZ=nz, H=h, DT=dt, Viscosity=0.0))
    e.SetAdvection(scheme)
    fu, fv = e.Mesh.U, e.Mesh.V
    gx = np.arange(fv.NX)  # V faces sit at cell centres in x: padded index i is x = (i - 1 + 0.5) h

    def profile(shift_cells):
        xc = gx - 1 + 0.5 - shift_cells
        row = np.sin(2 * math.pi * xc / cells_per_wave)
        return np.broadcast_to(row, (fv.NZ, fv.NY, fv.NX)).ravel().copy()

    v = profile(0.0)
    for _ in range(sweeps):
        e.upload("U", np.full(fu.NX * fu.NY * fu.NZ, u0))
        e.upload("V", v)
        e.upload("W", np.zeros(e.Mesh.W.NX * e.Mesh.W.NY * e.Mesh.W.NZ))
        e.sweep(0, dt)
        v = e.download("V")
    exact = profile(sweeps * 0.3)
    sel = np.zeros((fv.NZ, fv.NY, fv.NX), bool)
    sel[1:-1, 1:-1, 16:48] = True
    d = v.reshape(sel.shape)[sel] - exact.reshape(sel.shape)[sel]
    e.Close()
    return float(np.max(np.abs(d))), float(np.sqrt(np.mean(d * d)))


def test_maccormack_translates_a_wave_more_accurately():
    sl, sl_rms = translate_error(AF_ADVECTION_SEMI_LAGRANGIAN)
    mc, mc_rms = translate_error(AF_ADVECTION_MACCORMACK)
    print(f"error after 20 sweeps (max, rms): semi-Lagrangian {sl:.3e} {sl_rms:.3e}, "
          f"MacCormack {mc:.3e} {mc_rms:.3e}")
    assert sl > 0.1  # first-order damping of a 16-cell wave is large
    # The limiter reverts to the first-order value at the wave's extrema, so
    # the maximum error improves less than the mean.
    assert mc < 0.5 * sl
    assert mc_rms < 0.5 * sl_rms


def kinetic_energy_after(scheme, steps=20):
    c = Config(NX=32, NY=32, NZ=32, H=1 / 32, DT=0.004, Viscosity=1e-5, GaussSeidelIters=200)
    e = New(c)
    e.SeedDevice(1.0, 0.0, 42, 0)
    e.applyVelocityBC()
    e.SetAdvection(scheme)
    ke0 = e.KineticEnergy()
    e.Step(steps)
    ke, md = e.KineticEnergy(), e.MaxDivergence()
    e.Close()
    return ke0, ke, md


def test_vortex_loses_less_energy_with_maccormack():
    ke0, ke_sl, md_sl = kinetic_energy_after(AF_ADVECTION_SEMI_LAGRANGIAN)
    _, ke_mc, md_mc = kinetic_energy_after(AF_ADVECTION_MACCORMACK)
    print(f"KE {ke0:.6e} -> semi-Lagrangian {ke_sl:.6e}, MacCormack {ke_mc:.6e}; max|div| {md_sl:.2e} {md_mc:.2e}")
    assert math.isfinite(ke_mc) and ke_mc <= ke0 * 1.001
    assert ke_mc > ke_sl
    assert (ke0 - ke_mc) < 0.8 * (ke0 - ke_sl)


@pytest.mark.parametrize("shape,amp,nu", [((16, 16, 16), 1.0, 1e-5), ((24, 20, 18), 3.0, 1e-5),
                                          ((33, 17, 20), 1.0, 0.0), ((12, 10, 9), 25.0, 1e-5)])
def test_maccormack_steps_bit_exact(shape, amp, nu):
    # The oracle restates the MacCormack sweep in the kernel's binary64
    # operation order (forward step without diffusion, trace through phi^
    # with taps outside the written faces read from phi, limiter, diffusion
    # of phi): every sweep and whole Steps agree bit for bit, at amplitude 25
    # too (backtraces clamped at the walls), with and without viscosity.
    nx, ny, nz = shape
    c = Config(NX=nx, NY=ny, NZ=nz, H=1.0 / max(shape), DT=0.004, Viscosity=nu)
    gpu, orc = make_pair(c, "tg", amp, 0.01)
    gpu.SetAdvection(AF_ADVECTION_MACCORMACK)
    orc.set_advection(AF_ADVECTION_MACCORMACK)
    for axis in range(3):
        gpu.sweep(axis, 0.002)
        orc.sweep(axis, 0.002)
        assert_bit_identical(gpu, orc, ["U", "V", "W"], f"{shape} sweep {axis}")
    for k in range(2):
        gpu.Step(1)
        orc.step(1)
        assert_bit_identical(gpu, orc, ["U", "V", "W", "P", "Div"], f"{shape} step {k}")
    orc.close()


def test_switching_back_restores_bit_exact_parity():
    c = Config(NX=12, NY=10, NZ=9, H=1 / 12, DT=0.004, Viscosity=1e-5)
    gpu, orc = make_pair(c, "tg", 1.0, 0.01)
    gpu.SetAdvection(AF_ADVECTION_MACCORMACK)
    gpu.SetAdvection(AF_ADVECTION_SEMI_LAGRANGIAN)
    gpu.Step(3)
    orc.step(3)
    assert_bit_identical(gpu, orc, ["U", "V", "W", "P"], "after switching back")
    orc.close()


def test_rejections():
    e = New(Config(NX=8, NY=8, NZ=8, H=0.125, DT=0.005, Precision=AF_PRECISION_MIXED))
    with pytest.raises(AerofluxError):
        e.SetAdvection(AF_ADVECTION_MACCORMACK)
    e.SetAdvection(AF_ADVECTION_SEMI_LAGRANGIAN)  # the mixed form's own scheme
    e.Close()
    e = New(Config(NX=8, NY=8, NZ=8, H=0.125, DT=0.005))
    with pytest.raises(AerofluxError):
        e.SetAdvection(7)
    e.Close()


def test_nan_fault_keeps_the_reference_message():
    c = Config(NX=8, NY=8, NZ=8, H=0.125, DT=0.005)
    gpu, orc = make_pair(c, "vortex", 1.0, oracle_workers=1)
    gpu.SetAdvection(AF_ADVECTION_MACCORMACK)
    orc.set_advection(AF_ADVECTION_MACCORMACK)
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
    assert_bit_identical(gpu, orc, ["U", "V", "W", "P", "Div"], "state after fault")
    orc.close()
