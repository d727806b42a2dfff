"""af_kinetic_energy_noalloc: the entry point for callers that cannot
allocate device memory while they run (hosts that give all device memory to
their own pool up front, loops that cannot absorb cudaMalloc/cudaFree's
implicit device synchronisation).

It reads caller-owned device fields and keeps its scratch in a static device
array, so here the fields live in torch tensors (torch only as device-memory
plumbing) and its result is checked against the engine's own
af_kinetic_energy on the same field, within the relative 1e-12 the parity
tests allow KineticEnergy, on consecutive calls.  This file is collected last
so a failure here leaves every other test already run; it also passes alone
in a fresh process.
"""
import ctypes as C

import numpy as np
import pytest

from aeroflux_gb300 import _lib as L
from aeroflux_gb300 import Config, New
from aeroflux_gb300.workloads import taylor_green

pytestmark = pytest.mark.gpu

RTOL = 1e-12


def _stepped_engine(nx, ny, nz, steps=1):
    cfg = Config(NX=nx, NY=ny, NZ=nz, H=1.0 / max(nx, ny, nz), DT=0.002, Viscosity=1e-4, GaussSeidelIters=8)
    e = New(cfg)
    u, v, w = taylor_green(e.Cfg, 1.0, 0.01)
    for name, a in (("U", u), ("V", v), ("W", w)):
        e.upload(name, a)
    e.applyVelocityBC()
    e.Step(steps)
    return e


def _noalloc(cfg, tensors):
    import torch
    torch.cuda.synchronize()
    out = C.c_double(float("nan"))
    err = C.create_string_buffer(256)
    rc = L.lib().af_kinetic_energy_noalloc(C.byref(cfg.to_c()), tensors[0].data_ptr(), tensors[1].data_ptr(),
                                            tensors[2].data_ptr(), None, C.byref(out), err, 256)
    return rc, out.value, err.value.decode()


def _device_fields(e):
    import torch
    return [torch.from_numpy(e.download(n)).to("cuda:0") for n in ("U", "V", "W")]


def test_noalloc_kinetic_energy_matches_engine_on_consecutive_calls():
    e = _stepped_engine(40, 28, 33, steps=2)
    ref = e.KineticEnergy()
    fields = _device_fields(e)
    for call in range(2):
        rc, ke, msg = _noalloc(e.Cfg, fields)
        assert rc == L.AF_OK, msg
        assert abs(ke - ref) <= RTOL * abs(ref), f"call {call}: {ke!r} vs {ref!r}"
    # A smaller grid after a larger one: the shared array's stale partials
    # from the previous call must not leak into the result.
    e2 = _stepped_engine(17, 9, 12)
    ref2 = e2.KineticEnergy()
    rc, ke2, msg = _noalloc(e2.Cfg, _device_fields(e2))
    assert rc == L.AF_OK, msg
    assert abs(ke2 - ref2) <= RTOL * abs(ref2)
    e.Close()
    e2.Close()


def test_noalloc_rejects_grids_beyond_its_static_scratch():
    import torch
    cfg = Config(NX=2, NY=2, NZ=16385, Ghost=1, H=1.0)
    t = torch.zeros(8, dtype=torch.float64, device="cuda:0")
    out = C.c_double(0.0)
    err = C.create_string_buffer(256)
    rc = L.lib().af_kinetic_energy_noalloc(C.byref(cfg.to_c()), t.data_ptr(), t.data_ptr(), t.data_ptr(), None,
                                            C.byref(out), err, 256)
    assert rc == L.AF_ERR_ARG
    assert "at most 16384 z-planes" in err.value.decode()
    assert np.isfinite(out.value) and out.value == 0.0
