"""Serving: continuous batching of requests of different sizes.

Requests that arrive while others are on the GPU are admitted as slots and
memory free up and run in the same batched launches; each request's result
must be the same alone and in the mix (here: identical bits, tolerance 0).
"""
import numpy as np
import pytest

from aeroflux_gb300 import AF_PRECISION_MIXED, Config, New
from aeroflux_gb300.batch import Batch
from aeroflux_gb300.serve import Server, run_stream, run_stream_fp64
from aeroflux_gb300.workloads import served_requests, taylor_green
from tests.helpers import bits

pytestmark = pytest.mark.gpu


def req(nx, ny, nz, nu=2e-5):
    h = 1.0 / max(nx, ny, nz)
    return Config(NX=nx, NY=ny, NZ=nz, H=h, DT=min(0.004, 0.5 * h * h / (6 * nu)), Viscosity=nu, Density=1.0,
                  Precision=AF_PRECISION_MIXED, DivTol=1e-10)


REQS = [(req(32, 32, 32), 12), (req(48, 32, 16), 5), (req(16, 64, 32, 1e-4), 9), (req(32, 16, 48), 3),
        (req(64, 32, 32, 1e-6), 7), (req(16, 16, 80), 10), (req(48, 48, 32), 4), (req(32, 32, 64), 6)]


def padded_count(c, name):
    g = c.NX + 2, c.NY + 2, c.NZ + 2
    return {"U": (g[0] + 1) * g[1] * g[2], "V": g[0] * (g[1] + 1) * g[2], "W": g[0] * g[1] * (g[2] + 1)}[name]


def serve_all(reqs, max_slots, budget=8 << 30, round_steps=2):
    """Submits every request at once; results are downloaded and released as
    they finish (a retained result keeps its slot until released)."""
    srv = Server(budget, max_slots, 0, round_steps, retain=True)
    ids = [srv.submit(c, s) for c, s in reqs]
    cfg_of = dict(zip(ids, (c for c, _ in reqs)))
    done, fields = {}, {}
    rounds, max_resident = 0, 0
    while len(done) < len(ids):
        _, resident, _ = srv.round()
        max_resident = max(max_resident, resident)
        for r in srv.results():
            done[r["id"]] = r
            c = cfg_of[r["id"]]
            fields[r["id"]] = {n: srv.download(r["id"], n, padded_count(c, n)) for n in ("U", "V", "W")}
            srv.release(r["id"])
        rounds += 1
        assert rounds < 10000
    srv.close()
    return ids, done, fields, max_resident


def test_each_request_is_the_same_alone_and_in_the_mix():
    ids, done, mixed, max_res = serve_all(REQS, max_slots=3)
    assert max_res == 3  # requests overlapped on the device
    # Continuous batching: some request was admitted while another was running.
    rs = sorted(done.values(), key=lambda r: r["admitted_s"])
    assert any(b["admitted_s"] > a["admitted_s"] and b["admitted_s"] < a["completed_s"]
               for a in rs for b in rs if a is not b)
    for r in done.values():
        assert r["status"] == 0 and r["max_divergence"] <= 1e-10
        assert r["arrival_s"] <= r["admitted_s"] <= r["completed_s"]
    _, _, alone, max_res1 = serve_all(REQS, max_slots=1)
    assert max_res1 == 1
    for rid in ids:
        for n in ("U", "V", "W"):
            assert np.array_equal(bits(mixed[rid][n]), bits(alone[rid][n])), f"request {rid} field {n}"


def test_admission_respects_the_memory_budget():
    c = req(48, 48, 48)
    need = Batch.slot_bytes(c)
    srv = Server(2 * need + 8192, 16, 0, 2)  # budget for two requests
    for _ in range(5):
        srv.submit(c, 4)
    finished, rounds = 0, 0
    while finished < 5:
        _, resident, queued = srv.round()
        assert resident <= 2
        finished += len(srv.results())
        rounds += 1
        assert rounds < 1000
    srv.close()


def test_device_seed_matches_the_host_generator():
    c = req(24, 20, 28)
    e = New(c)
    e.SeedDevice(1.0, 0.01, 42, 7)
    u, v, w = taylor_green(e.Cfg, 1.0, 0.01, 42, 7)
    # W is noise only: identical bits (PCG32 jump-ahead on the device).
    assert np.array_equal(bits(e.download("W")), bits(w))
    # U, V add a binary32 Taylor-Green term: close to the host's libm values.
    assert np.max(np.abs(e.download("U") - u)) < 1e-6
    assert np.max(np.abs(e.download("V") - v)) < 1e-6
    e.Close()


def test_request_stream_summary():
    reqs = [(t, c, s) for t, c, s in served_requests(rate=20.0, duration=3.0, seed=5) if c.NX * c.NY * c.NZ < 2e6]
    out = run_stream(reqs, window=3.0, budget_bytes=16 << 30, max_slots=8, tune_after=4)
    print(out)
    assert out["completed_requests"] >= 1
    # Every offered request is either completed (admitted ones drain after
    # the window) or censored at its age when serving stopped.
    assert out["completed_requests"] + out["censored_requests"] == out["offered_requests"]
    assert out["p50_latency_s"] <= out["p99_latency_s"] <= out["elapsed_s"]
    assert out["worst_max_divergence"] <= 1e-10
    fp = run_stream_fp64(reqs, window=3.0, prepare=8)
    print(fp)
    assert fp["offered_requests"] == out["offered_requests"]
    assert fp["completed_requests"] + fp["censored_requests"] == fp["offered_requests"]


def test_requests_stop_after_their_own_steps_within_longer_rounds():
    # Rounds of up to 8 Steps while requests need 3..12: a request with fewer
    # Steps left than the round stops after its last one and matches a
    # standalone engine run for exactly its Steps.
    ids, done, served, _ = serve_all(REQS, max_slots=4, round_steps=8)
    for rid, (c, steps) in zip(ids, REQS):
        assert done[rid]["steps"] == steps
        e = New(c)
        e.SeedDevice(1.0, 0.01, 42, rid)
        e.applyVelocityBC()
        e.Step(steps)
        for n in ("U", "V", "W"):
            assert np.array_equal(bits(served[rid][n]), bits(e.download(n))), f"request {rid} field {n}"
        e.Close()
