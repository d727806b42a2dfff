"""The C ABI's error contract: every call reports misuse as a negative
af_status with an `aeroflux:` message (no exception, no crash, the engine
stays usable), calls on a closed engine answer AF_ERR_CLOSED, and an invalid
configuration fails with the reference's Normalize text
(aeroflux.go:47-113) on every entry point that takes one."""
import ctypes as C

import numpy as np
import pytest

from aeroflux_gb300 import AF_PRECISION_MIXED, AerofluxError, Config, New
from aeroflux_gb300 import _lib as L
from aeroflux_gb300.batch import Batch
from aeroflux_gb300.serve import Server

pytestmark = pytest.mark.gpu


def small(**kw):
    base = dict(NX=8, NY=6, NZ=5, H=0.125, DT=0.004, Viscosity=1e-4)
    base.update(kw)
    return Config(**base)


def last_error(e):
    return (L.lib().af_last_error(e._h) or b"").decode()


def test_bad_arguments_are_reported_and_the_engine_stays_usable():
    e = New(small())
    lib, h = L.lib(), e._h
    assert lib.af_step(h, -1) == L.AF_ERR_ARG and last_error(e) == "aeroflux: negative step count"
    assert lib.af_phase_sweep(h, 3, 0.001) == L.AF_ERR_ARG and last_error(e).startswith("aeroflux: axis")
    d = L.AfFieldDesc()
    assert lib.af_field_info(h, 8, C.byref(d)) == L.AF_ERR_ARG
    assert lib.af_field_info(h, -1, C.byref(d)) == L.AF_ERR_ARG
    n = e.Mesh.U.Count
    buf = np.zeros(n + 1)
    assert lib.af_field_upload(h, 1, buf.ctypes.data, n + 1) == L.AF_ERR_ARG
    assert last_error(e).startswith("aeroflux:")
    assert lib.af_field_download(h, 1, buf.ctypes.data, n - 1) == L.AF_ERR_ARG
    assert lib.af_field_upload(h, 9, buf.ctypes.data, n) == L.AF_ERR_ARG
    assert lib.af_max_divergence(h, None) == L.AF_ERR_ARG
    assert lib.af_step(None, 1) == L.AF_ERR_ARG
    # Still usable after all of that.
    e.Step(2)
    assert np.isfinite(e.MaxDivergence())
    e.Close()


def test_closed_engine_answers_closed():
    e = New(small())
    h = e._h
    lib = L.lib()
    assert lib.af_close(h) == L.AF_OK
    assert lib.af_close(h) == L.AF_OK  # idempotent (aeroflux.go:419-439)
    out = C.c_double()
    assert lib.af_step(h, 1) == L.AF_ERR_CLOSED
    assert lib.af_max_divergence(h, C.byref(out)) == L.AF_ERR_CLOSED
    assert (lib.af_last_error(h) or b"").decode() == "aeroflux: engine is closed"
    lib.af_destroy(h)
    e._h = None


@pytest.mark.parametrize("kw,msg", [
    (dict(NX=0), "aeroflux: interior extents must be positive, got 0x6x5"),
    (dict(Viscosity=-1.0), "aeroflux: viscosity must be finite and non-negative, got -1"),
    (dict(DT=1.0, Viscosity=1.0), "aeroflux: dt 1 exceeds explicit diffusion stability limit"),
])
def test_invalid_config_fails_with_the_reference_text_everywhere(kw, msg):
    cfg = small(**kw)
    with pytest.raises(AerofluxError) as ex:
        New(cfg)
    assert str(ex.value).startswith(msg)
    b = Batch(2)
    mixed = small(Precision=AF_PRECISION_MIXED, **kw)
    with pytest.raises(AerofluxError) as ex:
        b.assign(mixed)
    assert str(ex.value).startswith(msg)
    b.close()
    srv = Server(1 << 30, 4, 0, 2)
    with pytest.raises(AerofluxError) as ex:
        srv.submit(mixed, 3)
    assert str(ex.value).startswith(msg)
    srv.close()


def test_batch_misuse():
    b = Batch(1)
    s = b.assign(small(Precision=AF_PRECISION_MIXED))
    with pytest.raises(AerofluxError) as ex:
        b.assign(small(Precision=AF_PRECISION_MIXED))
    assert "full" in str(ex.value)
    lib = L.lib()
    buf = np.zeros(10)
    assert lib.af_batch_field_download(b._h, s + 5, 1, buf.ctypes.data, 10) == L.AF_ERR_ARG
    assert lib.af_batch_field_download(b._h, s, 1, buf.ctypes.data, 10) == L.AF_ERR_ARG  # wrong count
    assert lib.af_batch_step(b._h, -1) == L.AF_ERR_ARG
    b.step(1)
    assert b.max_divergence(s) <= 1e-10
    b.close()


def test_server_misuse():
    srv = Server(1 << 30, 2, 0, 2)
    lib = L.lib()
    rid = C.c_int64()
    cfg = small(Precision=AF_PRECISION_MIXED)
    assert lib.af_server_submit(srv._h, C.byref(cfg.to_c()), -3, 1, -1.0, C.byref(rid)) == L.AF_ERR_ARG
    buf = np.zeros(10)
    assert lib.af_server_download(srv._h, 12345, 1, buf.ctypes.data, 10) == L.AF_ERR_ARG
    assert lib.af_server_release(srv._h, 12345) == L.AF_ERR_ARG
    srv.close()
