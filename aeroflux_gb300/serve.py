"""Serving over the C ABI (af_server_*): continuous batching of simulation
requests of different sizes, admitted by device-memory budget, state resident
on the device, p50/p99 completion latency beside throughput.

run_stream() replays a request stream in real time against a server;
run_stream_fp64() serves the same stream with the plain FP64 engine, one
request at a time, as the comparison point.
"""
from __future__ import annotations

import ctypes as C
import time

import numpy as np

from . import _lib as L
from .engine import FIELD_IDS, AerofluxError, Config, New


class Server:
    def __init__(self, budget_bytes: int, max_slots: int = 32, device: int = 0, max_round_steps: int = 4,
                 retain: bool = False, max_resident_cells: int = 0):
        h = C.c_void_p()
        buf = C.create_string_buffer(512)
        rc = L.lib().af_server_create(budget_bytes, max_slots, max_resident_cells, device, max_round_steps,
                                      int(retain), C.byref(h), buf, 512)
        if rc != L.AF_OK:
            raise AerofluxError(buf.value.decode(), rc)
        self._h = h

    def _check(self, rc):
        if rc != L.AF_OK:
            raise AerofluxError((L.lib().af_server_last_error(self._h) or b"").decode(), rc)

    def now(self) -> float:
        t = C.c_double()
        self._check(L.lib().af_server_now(self._h, C.byref(t)))
        return t.value

    def submit(self, cfg: Config, steps: int, seed: int = 42, arrival: float = -1.0) -> int:
        i = C.c_int64()
        self._check(L.lib().af_server_submit(self._h, C.byref(cfg.to_c()), steps, seed, arrival, C.byref(i)))
        return i.value

    def round(self) -> tuple[int, int, int]:
        a, b, c = C.c_int64(), C.c_int64(), C.c_int64()
        self._check(L.lib().af_server_round(self._h, C.byref(a), C.byref(b), C.byref(c)))
        return a.value, b.value, c.value

    def results(self) -> list[dict]:
        buf = (L.AfRequestResult * 256)()
        out = []
        while True:
            n = C.c_int64()
            self._check(L.lib().af_server_results(self._h, buf, 256, C.byref(n)))
            for k in range(n.value):
                r = buf[k]
                out.append({f: getattr(r, f) for f, _ in L.AfRequestResult._fields_ if f != "reserved"})
            if n.value < 256:
                return out

    def download(self, rid: int, name: str, count: int) -> np.ndarray:
        a = np.empty(count)
        self._check(L.lib().af_server_download(self._h, rid, FIELD_IDS[name], a.ctypes.data, count))
        return a

    def release(self, rid: int) -> None:
        self._check(L.lib().af_server_release(self._h, rid))

    def cancel_queued(self) -> int:
        """Drops every request not yet admitted; returns how many."""
        n = C.c_int64()
        self._check(L.lib().af_server_cancel_queued(self._h, C.byref(n)))
        return n.value

    def stats(self) -> dict:
        s = L.AfServerStats()
        self._check(L.lib().af_server_get_stats(self._h, C.byref(s)))
        return {f: getattr(s, f) for f, _ in L.AfServerStats._fields_}

    def tune(self, reps: int = 3) -> str:
        buf = C.create_string_buffer(1 << 16)
        self._check(L.lib().af_server_tune(self._h, reps, buf, 1 << 16))
        return buf.value.decode()

    def close(self):
        if self._h:
            L.lib().af_server_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def _percentiles(x) -> tuple:
    if len(x) == 0:
        return None, None
    a = np.asarray(x, dtype=np.float64)
    return float(np.percentile(a, 50)), float(np.percentile(a, 99))


def _summary(done: list[dict], censored_ages: list[float], window: float, elapsed: float,
             offered_cell_steps: float, n_offered: int) -> dict:
    """Latency and throughput of a served stream.

    done: completed requests (arrival_s, completed_s relative to the stream
    start).  censored_ages: for every offered request that had not completed
    when serving stopped, its age at that moment (a lower bound of its
    latency).  p50/p99 over completed requests only are reported beside
    p50/p99 over ALL offered requests with the unfinished ones at their
    censored age -- a lower bound of the true percentiles that does not drop
    the requests the server could not take."""
    lat = [r["completed_s"] - r["arrival_s"] for r in done]
    p50, p99 = _percentiles(lat)
    a50, a99 = _percentiles(lat + list(censored_ages))
    served = float(sum(r["cells"] * r["steps"] for r in done))
    return {"window_s": window, "elapsed_s": elapsed, "offered_requests": n_offered,
            "completed_requests": len(done), "censored_requests": len(censored_ages),
            "p50_latency_s": p50, "p99_latency_s": p99,
            "p50_latency_all_offered_lower_bound_s": a50, "p99_latency_all_offered_lower_bound_s": a99,
            "completed_cell_steps_per_s": served / elapsed,
            "offered_cell_steps_per_s": offered_cell_steps / window,
            "worst_max_divergence": float(max((r["max_divergence"] for r in done), default=float("nan")))}


def run_stream(requests, window: float, budget_bytes: int = 150 << 30, max_slots: int = 128,
               max_round_steps: int = 8, device: int = 0, tune_after: int = 8,
               max_resident_cells: int = 96 << 20, drain: bool = True) -> dict:
    """Replays (arrival_s, cfg, steps) in real time: requests arrive for
    `window` seconds; afterwards nothing new is admitted and, with drain,
    the requests already resident step until they finish.  Requests still
    queued then are censored (reported with their count and age).

    The default caps (96 Mi resident cells, 128 slots, 8 Steps a round)
    trade latency for throughput: on GB300, over the 200/s benchmark stream
    (30 s windows), executed cell-steps/s rose from 0.83 G at 24 Mi cells,
    32 slots, 4 Steps a round to 0.93 G at 64 Mi, 0.97 G at 96 Mi and
    0.98 G at 128 Mi / 256 slots, while the median latency of completed
    requests rose from 21 s to 34 s (the stream is far beyond capacity, so
    queueing dominates latency at any cap)."""
    srv = Server(budget_bytes, max_slots, device, max_round_steps, max_resident_cells=max_resident_cells)
    pending = [r for r in requests if r[0] < window]
    offered = sum(c.NX * c.NY * c.NZ * s for _, c, s in pending)
    i, done, tuned = 0, [], False
    t0 = srv.now()
    while True:
        now = srv.now() - t0
        if now >= window:
            break
        while i < len(pending) and pending[i][0] <= now:
            a, cfg, steps = pending[i]
            srv.submit(cfg, steps, seed=42, arrival=t0 + a)
            i += 1
        fin, resident, queued = srv.round()
        if not tuned and (resident >= min(tune_after, max_slots) or srv.stats()["used_bytes"] > 0 and queued > 0):
            srv.tune(2)
            tuned = True
        done += srv.results()
        if resident == 0 and queued == 0 and i < len(pending):
            time.sleep(max(0.0, min(0.01, pending[i][0] - (srv.now() - t0))))
    # Cut-off: requests not yet admitted are cancelled and censored; with
    # drain, the resident ones step until they finish.
    st = srv.stats()
    queued_at_cutoff, resident_at_cutoff = st["queued"], st["resident"]
    cutoff = srv.now() - t0
    if drain:
        srv.cancel_queued()
        while srv.stats()["resident"] > 0:
            srv.round()
            done += srv.results()
    elapsed = srv.now() - t0
    st = srv.stats()
    srv.close()
    for r in done:
        r["arrival_s"] -= t0
        r["completed_s"] -= t0
        r["admitted_s"] -= t0
    # Request k (1-based) is pending[k-1]: the server numbers requests in
    # submission order and they are submitted in arrival order.
    finished = {r["id"] for r in done}
    stop = elapsed if drain else cutoff
    censored = [stop - a for k, (a, _, _) in enumerate(pending, start=1) if k not in finished]
    out = _summary(done, censored, window, elapsed, offered, len(pending))
    out.update({"executed_cell_steps_per_s": st["executed_cell_steps"] / elapsed, "cutoff_s": cutoff,
                "drain_s": elapsed - cutoff if drain else 0.0, "queued_at_cutoff": queued_at_cutoff,
                "resident_at_cutoff": resident_at_cutoff, "max_slots": max_slots, "budget_bytes": budget_bytes,
                "max_resident_cells": max_resident_cells, "max_round_steps": max_round_steps, "tuned": tuned})
    return out


def run_stream_fp64(requests, window: float, device: int = 0, chunk: int = 10, prepare: int = 160) -> dict:
    """The same stream served one request at a time by the plain FP64 engine
    (GaussSeidelIters at its default).  Engines for the first `prepare`
    requests are created before the stream starts (creation is setup, as in
    the reference's own benchmark), so the window times seeding and Steps;
    past those, engines are created in the window and counted.  After the
    window, the request in service finishes; the rest are censored."""
    pending = [r for r in requests if r[0] < window]
    offered = sum(c.NX * c.NY * c.NZ * s for _, c, s in pending)

    def make(cfg):
        c = Config(**{k: getattr(cfg, k) for k in ("NX", "NY", "NZ", "H", "DT", "Viscosity", "Density")},
                   Device=device)
        return New(c)

    ready = [make(cfg) for _, cfg, _ in pending[:prepare]]
    done, created_in_window = [], 0
    t0 = time.perf_counter()
    served = 0
    for rid, (arrival, cfg, steps) in enumerate(pending, start=1):
        now = time.perf_counter() - t0
        if now >= window:
            break
        if arrival > now:
            time.sleep(arrival - now)
        if rid - 1 < len(ready):
            e = ready[rid - 1]
        else:
            e = make(cfg)
            created_in_window += 1
        e.SeedDevice(1.0, 0.01, 42, rid)
        e.applyVelocityBC()
        left = steps
        while left > 0:
            k = min(chunk, left)
            e.Step(k)
            left -= k
        md = e.MaxDivergence()
        t = time.perf_counter() - t0
        served = rid
        done.append({"id": rid, "cells": cfg.NX * cfg.NY * cfg.NZ, "steps": steps, "arrival_s": arrival,
                     "completed_s": t, "max_divergence": md})
    elapsed = time.perf_counter() - t0
    for e in ready:
        e.Close()
    censored = [elapsed - a for a, _, _ in pending[served:]]
    out = _summary(done, censored, window, elapsed, offered, len(pending))
    out.update({"engines_created_before_window": len(ready), "engines_created_in_window": created_in_window})
    return out
