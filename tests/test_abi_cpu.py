"""C-ABI checks that need no GPU: the library loads, exports every symbol the
public header declares, and its host-side logic (Normalize, MACBytes, the
synthetic-input generator, error paths) matches the oracle."""
import ctypes as C
import math
import subprocess

import numpy as np
import pytest

from aeroflux_gb300 import _lib as L
from aeroflux_gb300 import AerofluxError, Config, MACBytes
from aeroflux_gb300.workloads import taylor_green
from oracle.oracle import go_format_float, mac_bytes, normalize


def test_library_exports_every_header_symbol():
    syms = L.header_symbols()
    assert "af_create" in syms and "af_step" in syms and len(syms) >= 25
    out = subprocess.run(["nm", "-D", "--defined-only", L.LIB_PATH], capture_output=True, text=True, check=True).stdout
    exported = {line.split()[-1] for line in out.splitlines() if " T " in line}
    missing = [s for s in syms if s not in exported]
    assert not missing, f"declared in include/aeroflux_cuda.h but not exported: {missing}"
    lib = L.lib()
    for s in syms:
        assert hasattr(lib, s)
    assert lib.af_abi_version() == 1


def test_signatures_cover_header():
    assert sorted(L.SIGNATURES) == L.header_symbols()


NORMALIZE_CASES = [
    dict(nx=16, ny=16, nz=16, workers=4),
    dict(nx=64, ny=64, nz=64, h=1 / 64, dt=0.004, viscosity=1e-5, workers=3),
    dict(nx=8, ny=8, nz=2, workers=64),
    dict(nx=12, ny=7, nz=5, ghost=2, viscosity=1e-3, workers=1),
    dict(nx=32, ny=32, nz=32, viscosity=2e-4, workers=2),            # DT default from viscosity
    dict(nx=0, ny=8, nz=8), dict(nx=-4, ny=8, nz=8), dict(nx=8, ny=8, nz=8, ghost=-1),
    dict(nx=8, ny=8, nz=8, viscosity=-1), dict(nx=8, ny=8, nz=8, h=math.nan),
    dict(nx=8, ny=8, nz=8, h=-math.inf), dict(nx=8, ny=8, nz=8, dt=math.inf),
    dict(nx=8, ny=8, nz=8, density=-2), dict(nx=8, ny=8, nz=8, h=0.1, viscosity=1.0, dt=1.0),
    dict(nx=8, ny=8, nz=8, workers=-3), dict(nx=8, ny=8, nz=8, gauss_seidel_iters=-1),
    dict(nx=256, ny=256, nz=256, h=1 / 256, viscosity=1e-5, dt=0.5),
    dict(nx=100, ny=100, nz=100, h=1e-7, viscosity=1e7, dt=1e300),
]
MAP = {"nx": "NX", "ny": "NY", "nz": "NZ", "ghost": "Ghost", "h": "H", "viscosity": "Viscosity",
       "density": "Density", "dt": "DT", "workers": "Workers", "gauss_seidel_iters": "GaussSeidelIters"}


@pytest.mark.parametrize("kw", NORMALIZE_CASES)
def test_normalize_matches_oracle(kw):
    ref, ref_err = normalize(**kw)
    cfg = Config(**{MAP[k]: v for k, v in kw.items()})
    err = None
    try:
        cfg.Normalize()
    except AerofluxError as e:
        err = str(e)
    assert err == ref_err
    if err is None:
        for k, py in MAP.items():
            assert getattr(cfg, py) == ref[k], k


def test_go_float_formatting_rules():
    # strconv 'g' shortest: %e from exponent >= 6 or < -4, two-digit exponent.
    cases = {0.1: "0.1", 1.0: "1", 1e6: "1e+06", 123456.0: "123456", 1234567.0: "1.234567e+06",
             1e-5: "1e-05", 0.0001: "0.0001", 0.01 / 6: "0.0016666666666666668", -2.0: "-2",
             math.inf: "+Inf", -math.inf: "-Inf", math.nan: "NaN", 1 / 64: "0.015625"}
    for v, want in cases.items():
        assert go_format_float(v) == want, v


def test_stability_message_text():
    cfg = Config(NX=8, NY=8, NZ=8, H=0.1, Viscosity=1.0, DT=1.0)
    with pytest.raises(AerofluxError) as ex:
        cfg.Normalize()
    assert str(ex.value) == ("aeroflux: dt 1 exceeds explicit diffusion stability limit 0.001666666666666667 "
                             "(h=0.1, nu=1); reduce dt or h")


@pytest.mark.parametrize("dims", [(1, 1, 1, 1), (8, 6, 4, 1), (64, 32, 16, 1), (12, 7, 5, 2), (256, 256, 256, 1)])
def test_mac_bytes_matches_oracle(dims):
    assert MACBytes(*dims) == mac_bytes(*dims)


def _pcg32_stream(seed, seq):
    mask = (1 << 64) - 1
    state, inc = 0, ((seq << 1) | 1) & mask

    def nxt():
        nonlocal state
        old = state
        state = (old * 6364136223846793005 + inc) & mask
        xs = (((old >> 18) ^ old) >> 27) & 0xFFFFFFFF
        rot = old >> 59
        return ((xs >> rot) | (xs << ((32 - rot) & 31))) & 0xFFFFFFFF

    nxt()
    state = (state + seed) & mask
    nxt()
    while True:
        a, b = nxt() >> 5, nxt() >> 6
        yield (a * 67108864.0 + b) * (1.0 / 9007199254740992.0)


def test_taylor_green_generator_matches_restatement():
    """af_seed_taylor_green against a pure-Python restatement (math.sin is the
    same libm the library calls on this host)."""
    cfg = Config(NX=6, NY=5, NZ=4, H=1 / 6, DT=0.001)
    cfg.Normalize()
    amp, noise = 1.0, 0.01
    u, v, w = taylor_green(cfg, amp, noise, seed=42, stream=3)
    g, NX, NY, NZ, h = 1, 6, 5, 4, cfg.H
    cx, cy, cz = NX + 2, NY + 2, NZ + 2
    ru, rv, rw = np.zeros((cx + 1) * cy * cz), np.zeros(cx * (cy + 1) * cz), np.zeros(cx * cy * (cz + 1))
    rng = _pcg32_stream(42, 3)
    tp = 6.283185307179586
    for z in range(g, g + NZ):
        for y in range(g, g + NY):
            for x in range(g, g + NX + 1):
                X, Y, Z = (x - g) * h, ((y - g) + 0.5) * h, ((z - g) + 0.5) * h
                ru[x + y * (cx + 1) + z * (cx + 1) * cy] = amp * math.sin(tp * X) * math.cos(tp * Y) * math.cos(tp * Z) + noise * (2.0 * next(rng) - 1.0)
    for z in range(g, g + NZ):
        for y in range(g, g + NY + 1):
            for x in range(g, g + NX):
                X, Y, Z = ((x - g) + 0.5) * h, (y - g) * h, ((z - g) + 0.5) * h
                rv[x + y * cx + z * cx * (cy + 1)] = -amp * math.cos(tp * X) * math.sin(tp * Y) * math.cos(tp * Z) + noise * (2.0 * next(rng) - 1.0)
    for z in range(g, g + NZ + 1):
        for y in range(g, g + NY):
            for x in range(g, g + NX):
                rw[x + y * cx + z * cx * cy] = 0.0 + noise * (2.0 * next(rng) - 1.0)
    for a, b in ((u, ru), (v, rv), (w, rw)):
        assert np.array_equal(a.view(np.uint64), b.view(np.uint64))


def test_pcg32_reference_vector():
    # pcg32_srandom_r(42, 54) first outputs, from the PCG reference demo (pcg32-demo.c).
    mask = (1 << 64) - 1
    state, inc = 0, (54 << 1) | 1

    def nxt():
        nonlocal state
        old = state
        state = (old * 6364136223846793005 + inc) & mask
        xs = (((old >> 18) ^ old) >> 27) & 0xFFFFFFFF
        rot = old >> 59
        return ((xs >> rot) | (xs << ((32 - rot) & 31))) & 0xFFFFFFFF

    nxt()
    state = (state + 42) & mask
    nxt()
    assert [nxt() for _ in range(6)] == [0xa15c02b7, 0x7b47f409, 0xba1d3330, 0x83d2f293, 0xbfa4784b, 0xcbed606e]


def test_create_without_device_fails_cleanly():
    import torch
    if torch.cuda.is_available():
        pytest.skip("a device is present")
    c = Config(NX=8, NY=8, NZ=8).to_c()
    h = C.c_void_p()
    buf = C.create_string_buffer(512)
    rc = L.lib().af_create(C.byref(c), C.byref(h), buf, 512)
    assert rc in (L.AF_ERR_CUDA, L.AF_ERR_NOMEM) and not h.value
    assert buf.value.decode().startswith("aeroflux: ")


def test_batch_slot_rejects_grids_beyond_its_32_bit_index_space():
    """A thin wide grid whose fields fit 2^31 elements but whose velocity-BC
    write set does not (about 2.4e9 ghost cells at 20000x20000x1) is refused
    before any device work, as is a field beyond 2^31 elements."""
    from aeroflux_gb300 import _lib as LL
    from aeroflux_gb300.batch import Batch
    ok = Config(NX=64, NY=48, NZ=32, H=1 / 64, DT=0.001, Precision=LL.AF_PRECISION_MIXED)
    assert Batch.slot_bytes(ok) > 0
    for dims in ((20000, 20000, 1), (1300, 1300, 1300)):
        c = Config(NX=dims[0], NY=dims[1], NZ=dims[2], H=1 / max(dims), DT=1e-9, Viscosity=1e-5,
                   Precision=LL.AF_PRECISION_MIXED)
        with pytest.raises(AerofluxError):
            Batch.slot_bytes(c)


def test_oracle_seeder_matches_the_product_generator():
    """The reference arm of the benchmark seeds through the oracle alone; its
    field is the product generator's bit for bit (same host libm)."""
    from oracle.oracle import OracleEngine
    cfg = Config(NX=9, NY=7, NZ=5, H=1 / 9, DT=0.001)
    cfg.Normalize()
    u, v, w = taylor_green(cfg, 1.0, 0.01, seed=42, stream=2)
    with OracleEngine(nx=9, ny=7, nz=5, h=1 / 9, dt=0.001, viscosity=0.0, density=1.0) as o:
        o.seed_taylor_green(1.0, 0.01, 42, 2)
        for fid, a in ((1, u), (2, v), (3, w)):
            assert np.array_equal(o.data(fid).view(np.uint64), a.view(np.uint64))
