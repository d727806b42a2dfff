"""The served stream's summary (host logic of aeroflux_gb300.serve): latency
percentiles over completed requests and, as a lower bound, over every offered
request with the unfinished ones at their censored age; throughput over the
elapsed time; nothing is dropped from the counts."""
import math

import numpy as np

from aeroflux_gb300.serve import _summary


def req(arrival, completed, cells=1000, steps=10, max_div=1e-11):
    return {"arrival_s": arrival, "completed_s": completed, "cells": cells, "steps": steps,
            "max_divergence": max_div}


def test_percentiles_and_throughput():
    done = [req(0.0, 1.0), req(0.5, 3.5), req(1.0, 2.0, cells=2000, max_div=3e-11)]
    out = _summary(done, [10.0, 12.0], window=4.0, elapsed=5.0, offered_cell_steps=9e4, n_offered=5)
    lat = [1.0, 3.0, 1.0]
    assert math.isclose(out["p50_latency_s"], float(np.percentile(lat, 50)))
    assert math.isclose(out["p99_latency_s"], float(np.percentile(lat, 99)))
    every = lat + [10.0, 12.0]
    assert math.isclose(out["p50_latency_all_offered_lower_bound_s"], float(np.percentile(every, 50)))
    assert math.isclose(out["p99_latency_all_offered_lower_bound_s"], float(np.percentile(every, 99)))
    assert out["completed_requests"] == 3 and out["censored_requests"] == 2 and out["offered_requests"] == 5
    assert math.isclose(out["completed_cell_steps_per_s"], (1000 * 10 * 2 + 2000 * 10) / 5.0)
    assert math.isclose(out["offered_cell_steps_per_s"], 9e4 / 4.0)
    assert out["worst_max_divergence"] == 3e-11


def test_censored_requests_raise_the_lower_bound():
    # With most requests unfinished, the percentiles over every offered
    # request sit at or above those of the completed ones.
    done = [req(0.0, 0.5), req(0.1, 0.7)]
    out = _summary(done, [30.0] * 20, window=30.0, elapsed=31.0, offered_cell_steps=1e9, n_offered=22)
    assert out["p99_latency_all_offered_lower_bound_s"] >= out["p99_latency_s"]
    assert out["p50_latency_all_offered_lower_bound_s"] == 30.0


def test_nothing_completed():
    out = _summary([], [5.0, 6.0], window=2.0, elapsed=6.0, offered_cell_steps=1e6, n_offered=2)
    assert out["completed_requests"] == 0 and out["censored_requests"] == 2
    assert out["completed_cell_steps_per_s"] == 0.0
    assert math.isnan(out["worst_max_divergence"])
