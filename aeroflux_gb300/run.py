"""Runs one cubic workload through the engine and prints a JSON summary.

    python -m aeroflux_gb300.run --n 256 --steps 2 [--gsi 200] [--dt 0.001] [--nu 1e-5]
                                 [--precision fp64|mixed] [--project N] [--inner-sweeps K] [--warmup W]
                                 [--multigrid TOL] [--maccormack] [--batch G] [--profile-range]
                                 [--tune-report]

--project N runs N projections (BC, divergence, red-black sweeps, gradient)
instead of Steps.  The initial field is the seeded Taylor-Green vortex with
uniform noise used by the benchmark.  --batch G steps the first G grids of
the batched workload (extents from {32,48,64,96,128}, mixed form) in one
tuned batch instead of one cube.  --profile-range brackets the measured
Steps (not the set-up, tuning or warm-up) with the CUDA profiler's start and
stop, for `ncu --profile-from-start off`.  --tune-report prints the
autotuner's report instead of stepping (the batch's, or that of a one-slot
batch holding the mixed-form cube): the chosen launch shape of every stage
and, for the fused red-black pair stages, every tile variant's time.
"""
from __future__ import annotations

import argparse
import contextlib
import json
import time

from . import AF_ADVECTION_MACCORMACK, AF_PRECISION_FP64, AF_PRECISION_MIXED, Config, New
from .workloads import taylor_green


@contextlib.contextmanager
def profiler_range(on: bool):
    """cudaProfilerStart/Stop around the block (through torch's CUDA runtime)."""
    if not on:
        yield
        return
    import torch
    torch.cuda.synchronize()
    torch.cuda.profiler.start()
    try:
        yield
    finally:
        torch.cuda.synchronize()
        torch.cuda.profiler.stop()


def run_batch(a) -> None:
    from .batch import Batch
    from .workloads import batched_instances
    cfgs = batched_instances(a.batch)
    b = Batch(len(cfgs))
    slots = [b.assign(c) for c in cfgs]
    rep = b.tune(5 if a.tune_report else 2)
    if a.tune_report:
        print(json.dumps(rep))
        b.close()
        return
    for s in slots:
        b.seed(s, 1.0, a.noise, 42, s)
    b.apply_velocity_bc()
    if a.warmup:
        b.step(a.warmup)
    t0 = time.perf_counter()
    with profiler_range(a.profile_range):
        b.step(a.steps)
    dt = time.perf_counter() - t0
    cells = sum(c.NX * c.NY * c.NZ for c in cfgs)
    print(json.dumps({"grids": len(cfgs), "cells": cells, "steps": a.steps, "seconds": dt,
                      "cell_steps_per_s": cells * a.steps / dt,
                      "worst_max_divergence": max(b.max_divergence(s) for s in slots)}))
    b.close()


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--n", type=int, default=64)
    ap.add_argument("--steps", type=int, default=1)
    ap.add_argument("--gsi", type=int, default=200)
    ap.add_argument("--dt", type=float, default=0.001)
    ap.add_argument("--nu", type=float, default=1e-5)
    ap.add_argument("--noise", type=float, default=0.01)
    ap.add_argument("--precision", choices=["fp64", "mixed"], default="fp64")
    ap.add_argument("--project", type=int, default=0)
    ap.add_argument("--inner-sweeps", type=int, default=0)
    ap.add_argument("--warmup", type=int, default=0, help="untimed Steps (or projections) first")
    ap.add_argument("--maccormack", action="store_true", help="FP64 form with MacCormack advection")
    ap.add_argument("--multigrid", type=float, default=None, metavar="TOL",
                    help="FP64 form with the multigrid projection to max|div| <= TOL (0: 1e-12)")
    ap.add_argument("--batch", type=int, default=0, help="step the first G grids of the batched workload")
    ap.add_argument("--profile-range", action="store_true",
                    help="bracket the measured Steps with cudaProfilerStart/Stop")
    ap.add_argument("--tune-report", action="store_true", help="print the autotuner's report and exit")
    a = ap.parse_args()
    if a.batch:
        run_batch(a)
        return
    if a.tune_report:
        from .batch import Batch
        b = Batch(1)
        s = b.assign(Config(NX=a.n, NY=a.n, NZ=a.n, H=1.0 / a.n, DT=a.dt, Viscosity=a.nu, Density=1.0,
                            Precision=AF_PRECISION_MIXED, InnerSweeps=a.inner_sweeps))
        b.seed(s, 1.0, a.noise, 42, 0)
        print(json.dumps(b.tune(5)))
        b.close()
        return
    prec = AF_PRECISION_MIXED if a.precision == "mixed" else AF_PRECISION_FP64
    cfg = Config(NX=a.n, NY=a.n, NZ=a.n, H=1.0 / a.n, DT=a.dt, Viscosity=a.nu, Density=1.0,
                 GaussSeidelIters=a.gsi, Precision=prec, InnerSweeps=a.inner_sweeps)
    e = New(cfg)
    u, v, w = taylor_green(e.Cfg, 1.0, a.noise)
    e.upload("U", u)
    e.upload("V", v)
    e.upload("W", w)
    e.applyVelocityBC()
    if a.multigrid is not None:
        e.EnableMultigridSolver(a.multigrid)
    if a.maccormack:
        e.SetAdvection(AF_ADVECTION_MACCORMACK)
    for _ in range(a.warmup):
        e.project() if a.project else e.Step(1)
    t0 = time.perf_counter()
    with profiler_range(a.profile_range):
        if a.project:
            for _ in range(a.project):
                e.project()
            n = a.project
        else:
            e.Step(a.steps)
            n = a.steps
    dt = time.perf_counter() - t0
    out = {"n": a.n, "precision": a.precision, "calls": n, "what": "project" if a.project else "step",
           "seconds": dt, "cell_steps_per_s": a.n ** 3 * n / dt, "max_divergence": e.MaxDivergence()}
    if prec == AF_PRECISION_MIXED or a.multigrid is not None:
        out["refinement_passes"] = e.LastProjectionStats()[0]
    print(json.dumps(out))
    e.Close()


if __name__ == "__main__":
    main()
