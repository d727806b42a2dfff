#!/usr/bin/env python3
"""Throughput benchmark of the fractional-step Step on GB300.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Workload (one "step" = one Step of the engine): a single 256^3 MAC grid in
binary64, H=1/256, DT=0.001, Viscosity=1e-5, 200 red-black sweep pairs per
projection, Taylor-Green vortex (amplitude 1) plus seeded uniform +-0.01
PCG32 noise.  Metric: interior cell-steps per second (NX*NY*NZ*steps/s, the
reference's Mcell/s of bench_test.go:32).

ours: `value` is device time (CUDA event nodes carried by the step graph on
the engine's stream) over exactly K steps with the field resident in HBM; the
working set (1.1 GB per grid) is far larger than L2.  `e2e` times the same
step through the C ABI as a Mesh.Data caller sees it: U, V, W uploaded from
pinned host memory, Step, MaxDivergence read back and U, V, W downloaded,
every step.  `roofline` is the
red-black sweep kernel, the dominant one.  `cpu_baseline` times the CPU
oracle (a C restatement of the reference's Go CPU path) on a bounded sample.

reference: the reference's CPU algorithm (the oracle, since Go is not
available) on all host cores, W + K steps of the same workload.

N > 1 runs independent replicas (the path has no exchange step): one grid per
GPU, no collective on the data path; the barrier and max-over-ranks timing
use a gloo process group.
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "cell-steps/s at 256^3 (FP64 vs mixed, same div tol); served p50/p99 latency"
UNIT = "cell-steps/s"
N = 256
DT = 0.001
NU = 1e-5
GSI = 200
NOISE = 0.01
WORKLOAD = f"plain-fp64 {N}^3 MAC grid, H=1/{N}, DT={DT}, Viscosity={NU}, {GSI} red-black pairs/projection"
HBM_FALLBACK_GBS = 6800.0


def rank_info():
    return (int(os.environ.get("RANK", 0)), int(os.environ.get("LOCAL_RANK", 0)),
            int(os.environ.get("WORLD_SIZE", 1)))


class Dist:
    """Barrier / max-reduce across replica ranks (gloo; nothing on the data path)."""

    def __init__(self, world):
        self.world = world
        if world > 1:
            import torch.distributed as dist
            dist.init_process_group("gloo")
            self.d = dist

    def barrier(self):
        if self.world > 1:
            self.d.barrier()

    def max(self, x: float) -> float:
        if self.world == 1:
            return x
        import torch
        t = torch.tensor([x], dtype=torch.float64)
        self.d.all_reduce(t, op=self.d.ReduceOp.MAX)
        return float(t.item())

    def close(self):
        if self.world > 1:
            self.d.destroy_process_group()


class ClockSampler:
    """nvidia-smi clocks and throttle reasons, sampled during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.idx = gpu_index
        self.proc = None
        self.f = None

    def start(self):
        try:
            self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                                          "-lms", "200"], stdout=self.f, stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None

    def stop(self) -> dict:
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.f.flush()
        self.f.seek(0)
        text = self.f.read()
        self.f.close()
        os.unlink(self.f.name)
        return parse_clocks(text, self.idx)


def parse_clocks(text: str, gpu_index: int) -> dict:
    """Median SM clock, maximum clock and the throttle reasons seen in the
    sampler's CSV (ClockSampler.Q, no header, no units); with several GPUs
    in the samples, only gpu_index's rows count."""
    rows = [r.split(",") for r in text.strip().splitlines() if r.strip()]
    rows = [[c.strip() for c in r] for r in rows if len(r) >= 9]
    ids = {r[0] for r in rows}
    if len(ids) > 1:
        rows = [r for r in rows if r[0] == str(gpu_index)]
    sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
    mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
    names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
    reasons = sorted({names[k] for r in rows for k in range(4) if r[5 + k].lower() == "active"})
    return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
            "reasons": reasons, "samples": len(rows)}


def measured_peaks() -> tuple[float, str]:
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(p) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return HBM_FALLBACK_GBS, "fallback"


def profiled_traffic(name: str) -> float | None:
    """DRAM bytes per launch from a committed ncu summary (profiles/<name>.md,
    line `dram_bytes_per_launch: <int>`), or None."""
    p = os.path.join(ROOT, "profiles", name + ".md")
    try:
        for line in open(p):
            if line.strip().startswith("dram_bytes_per_launch:"):
                return float(line.split(":", 1)[1].strip().split()[0])
    except OSError:
        pass
    return None


def cpu_threads() -> int:
    try:
        return len(os.sched_getaffinity(0))
    except AttributeError:
        return os.cpu_count() or 1


def base_config():
    from aeroflux_gb300.workloads import PLAIN_256
    return PLAIN_256


def run_oracle_steps(warmup: int, steps: int, threads: int):
    """The CPU path (oracle) on the same workload: seconds per step.  The
    input is seeded by the oracle itself (the same Taylor-Green + PCG32
    field), so this path maps no product code."""
    from oracle.oracle import OracleEngine
    with OracleEngine(nx=N, ny=N, nz=N, h=1.0 / N, dt=DT, viscosity=NU, density=1.0,
                      gauss_seidel_iters=GSI, workers=threads) as o:
        o.seed_taylor_green(1.0, NOISE, 42, 0)
        o.apply_velocity_bc()
        for _ in range(warmup):
            o.step()
        t0 = time.perf_counter()
        for _ in range(steps):
            o.step()
        return (time.perf_counter() - t0) / max(steps, 1)


def common_fields(args, world):
    return {
        "metric": METRIC, "unit": UNIT, "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic: Taylor-Green vortex amplitude 1 + uniform +-0.01 PCG32 noise (seed 42, stream=rank)",
        "config": {"workload": WORKLOAD, "grid": [N, N, N], "dt": DT, "viscosity": NU, "gauss_seidel_iters": GSI,
                   "precision": "fp64 (bit-identical to the CPU path)",
                   "l2": "inputs larger than L2: 1.10 GB arena per grid vs 129 MB L2",
                   "parallelism": f"replicas x{world} (one grid per GPU, no collective)"},
    }


def product_library_mapped() -> bool:
    """Whether this process has mapped the product's CUDA library."""
    try:
        with open("/proc/self/maps") as f:
            return any("libaeroflux_cuda" in line for line in f)
    except OSError:
        return False


def bench_reference(args):
    rank, _, world = rank_info()
    if rank != 0:
        return 0
    threads = cpu_threads()
    sec = run_oracle_steps(args.warmup, args.steps, threads)
    if product_library_mapped():
        raise RuntimeError("the reference arm mapped the product library")
    val = N ** 3 / sec
    line = common_fields(args, world)
    line.update({
        "impl": "reference", "value": val, "ms_per_step": sec * 1e3, "product_library_mapped": False,
        "cpu_baseline": {"value": val, "unit": UNIT, "cores": threads, "kind": "port",
                         "sample": f"{args.warmup} warm-up + {args.steps} timed Steps of the {N}^3 workload, "
                                   f"C restatement of the Go CPU path, {threads} worker threads"},
        "e2e": {"value": val, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    })
    print(json.dumps(line), flush=True)
    return 0


def mixed_bytes_per_cell_step(passes: float, vcycles: float, nu: int = 2) -> float:
    """Algorithmic bytes per cell-step of the mixed form at its stored widths
    (binary64 state, binary32 multigrid), for a projection of `passes`
    refinement passes and `vcycles` V-cycles in all: six sweeps (read U, V,
    W, write three faces: 48 B); per projection the divergence (read U, V,
    W, write Div: 32 B), the first residual (read p, B, write r, zero e:
    24 B), per pass the correction (read p, e, write p: 20 B) and the
    residual (24 B), per V-cycle (per level cell) 2*nu fused red-black pairs
    of 12 B, restriction 9 B and prolongation 8.5 B, the coarser levels
    adding 1/7, and the gradient (read p, read and write U, V, W: 56 B)."""
    vcycle = (2 * nu * 12 + 9 + 8.5) * 8 / 7
    return 6 * 48 + 2 * (32 + 24 + passes * 44 + vcycles * vcycle + 56)


def new_engine(precision: int, local: int, rank: int, div_tol: float = 0.0):
    from aeroflux_gb300 import New
    from aeroflux_gb300.workloads import taylor_green
    cfg = base_config().config(Device=local, Precision=precision, DivTol=div_tol)
    e = New(cfg)
    u, v, w = taylor_green(e.Cfg, 1.0, NOISE, 42, rank)
    for name, a in (("U", u), ("V", v), ("W", w)):
        e.upload(name, a)
    e.applyVelocityBC()
    return e, (u, v, w)


def velocity_host(e):
    return [e.download(n) for n in ("U", "V", "W")]


def error_vs_fp64(mixed_fields, ref_engine, md_mixed: float, steps: int) -> dict:
    """max|dU,dV,dW| / max|ref| of the mixed form against the FP64 form with
    the multigrid projection (bit-exact FP64 sweeps, max|div| <= 1e-12),
    both from the same field after the same Steps."""
    out = {"reference": "FP64 form + EnableMultigridSolver(1e-12), same initial field and Steps",
           "steps": steps, "max_divergence_mixed": md_mixed, "max_divergence_fp64": ref_engine.MaxDivergence()}
    for name, a in zip(("U", "V", "W"), mixed_fields):
        b = ref_engine.download(name)
        out[f"rel_{name}"] = float(abs(a - b).max() / max(abs(b).max(), 1e-300))
    out["rel_max"] = max(out["rel_U"], out["rel_V"], out["rel_W"])
    return out


def device_timed(e, steps: int, warmup: int, dist, clocks=None):
    """Exactly `steps` Steps timed by the step graph's event nodes (device
    time on the engine's stream), after `warmup` untimed Steps."""
    e.Profile(True)
    for _ in range(warmup):
        e.Step(1)
    dist.barrier()
    if clocks:
        clocks.start()
        time.sleep(0.3)
    dev_ms = solve_ms = sw_ms = 0.0
    passes, vcyc = [], []
    t0 = time.perf_counter()
    prof = None
    for _ in range(steps):
        e.Step(1)  # synchronous: returns after the step graph completes
        prof = e.LastStepProfile()
        dev_ms += prof.step_ms
        solve_ms += prof.rbgs_ms
        sw_ms += prof.sweep_ms
        passes.append(e.LastProjectionStats()[0])
        vcyc.append(e.LastProjectionVCycles())
    wall = time.perf_counter() - t0
    clk = clocks.stop() if clocks else None
    dist.barrier()
    e.Profile(False)
    return {"dev_s": dist.max(dev_ms / 1e3), "wall_s": wall, "solve_ms": solve_ms / steps, "sweep_ms": sw_ms / steps,
            "launches": prof.kernel_launches, "rbgs_launches": prof.rbgs_launches, "passes": passes, "vcycles": vcyc,
            "clocks": clk}


def bench_mixed_512(args, dist, local, rank):
    """512^3 mixed-precision config: DT=0.0005, noise 0.05, max|div| <= 1e-10."""
    from aeroflux_gb300 import New
    from aeroflux_gb300.workloads import MIXED_512
    e = New(MIXED_512.config(Device=local, DivTol=1e-10))
    e.SeedDevice(1.0, MIXED_512.noise, 42, rank)
    e.applyVelocityBC()
    steps = max(2, args.steps // 2)
    t = device_timed(e, steps, 1, dist)
    n = MIXED_512.n ** 3
    md = e.MaxDivergence()
    out = {"value": n * steps * dist.world / t["dev_s"], "unit": UNIT, "steps": steps,
           "ms_per_step": t["dev_s"] * 1e3 / steps, "max_divergence_after": md,
           "refinement_passes_last_projection": t["passes"],
           "stages_ms_per_step": {"projections": t["solve_ms"], "sweeps": t["sweep_ms"]},
           "workload": MIXED_512.name}
    fields = velocity_host(e)
    e.Close()
    # The same field and Steps in the FP64 form with the exact projection.
    from aeroflux_gb300 import _lib as L
    ref = New(MIXED_512.config(Device=local, Precision=L.AF_PRECISION_FP64))
    ref.SeedDevice(1.0, MIXED_512.noise, 42, rank)
    ref.applyVelocityBC()
    ref.EnableMultigridSolver(1e-12)
    ref.Step(1 + steps)
    out["error_vs_fp64"] = error_vs_fp64(fields, ref, md, 1 + steps)
    ref.Close()
    return out


def bench_batched(args, dist, local):
    """256 uneven grids, one persistent launch per stage, one graph per step."""
    from aeroflux_gb300 import New
    from aeroflux_gb300.batch import Batch
    from aeroflux_gb300.workloads import batched_instances
    cfgs = batched_instances(256)
    b = Batch(len(cfgs), device=local)
    slots = [b.assign(c) for c in cfgs]
    t0 = time.perf_counter()
    tune = b.tune(3)
    tune_s = time.perf_counter() - t0
    for s in slots:
        b.seed(s, 1.0, 0.01, 42, s)
    b.apply_velocity_bc()
    cells = sum(c.NX * c.NY * c.NZ for c in cfgs)
    steps = args.steps
    for _ in range(args.warmup):
        b.step(1)
    b.profile(True)
    dev_ms = sw = pj = 0.0
    dist.barrier()
    for _ in range(steps):
        b.step(1)
        p = b.last_step_profile()
        dev_ms += p.step_ms
        sw += p.sweep_ms
        pj += p.rbgs_ms
    dev_s = dist.max(dev_ms / 1e3)
    worst = max(b.max_divergence(s) for s in slots)
    passes = max(b.projection_stats(s)[0] for s in slots)
    b.close()
    value = cells * steps * dist.world / dev_s
    # The plain FP64 form on the same mixed-size workload: a stratified
    # sample (every fourth grid of the generator's order, 64 grids), each
    # alone, 10 timed Steps after one warm-up (GaussSeidelIters at its
    # default); the aggregate is sampled cells x steps / sampled time.
    sample = cfgs[::4]
    k = 10
    tot_cells_steps, tot_s, divs = 0, 0.0, []
    for i, c in enumerate(sample):
        cf = type(c)(**{kk: getattr(c, kk) for kk in ("NX", "NY", "NZ", "H", "DT", "Viscosity", "Density")},
                     Device=local)
        e = New(cf)
        e.SeedDevice(1.0, 0.01, 42, i)
        e.applyVelocityBC()
        e.Step(1)
        e.Profile(True)
        ms = 0.0
        for _ in range(k):
            e.Step(1)
            ms += e.LastStepProfile().step_ms
        tot_cells_steps += c.NX * c.NY * c.NZ * k
        tot_s += ms / 1e3
        divs.append(e.MaxDivergence())
        e.Close()
    plain = tot_cells_steps / tot_s
    return {"value": value, "unit": UNIT, "instances": len(cfgs), "cells": cells, "steps": steps,
            "ms_per_step": dev_s * 1e3 / steps, "stages_ms_per_step": {"sweeps": sw / steps, "projections": pj / steps},
            "worst_max_divergence_after": worst, "max_refinement_passes_last_projection": passes,
            "autotune_s": tune_s, "autotuned_stages": len(tune),
            "plain_fp64_same_workload": {"value": plain, "unit": UNIT, "sample_grids": len(sample),
                                         "sample": "every fourth grid, 10 timed Steps each",
                                         "worst_max_divergence_after": max(divs),
                                         "gauss_seidel_iters": 24},
            "speedup_vs_plain_fp64": value / plain,
            "workload": "256 grids, extents from {32,48,64,96,128} by PCG32 seed, H=1/max, nu log-uniform "
                        "[1e-6,1e-4], DT=min(0.004, 0.5H^2/(6nu)), mixed form, div tol 1e-10"}


def bench_served(args, local):
    from aeroflux_gb300.serve import run_stream, run_stream_fp64
    from aeroflux_gb300.workloads import served_requests
    reqs = served_requests(200.0, args.serve_seconds, 42)
    mixed = run_stream(reqs, args.serve_seconds, budget_bytes=150 << 30, max_slots=128, max_round_steps=8,
                       max_resident_cells=96 << 20, device=local)
    fp64 = run_stream_fp64(reqs, args.serve_seconds, device=local)
    return {"mixed": mixed, "plain_fp64_sequential": fp64,
            "workload": f"Poisson arrivals at 200/s for {args.serve_seconds:g} s, extents uniform over multiples "
                        "of 16 in [32,192], steps uniform in [50,500], 150 GB budget; after the arrivals end, "
                        "requests not yet admitted are censored and the resident ones finish",
            "completed_throughput_ratio": (mixed["completed_cell_steps_per_s"] /
                                           max(fp64["completed_cell_steps_per_s"], 1e-30))}


def bench_ours(args):
    from aeroflux_gb300 import _lib as L

    rank, local, world = rank_info()
    dist = Dist(world)
    cells = N ** 3

    # --- plain FP64 (the headline workload) ---------------------------------
    e, (u, v, w) = new_engine(L.AF_PRECISION_FP64, local, rank)
    t = device_timed(e, args.steps, args.warmup, dist, ClockSampler(local))
    value = cells * args.steps * world / t["dev_s"]
    md_plain = e.MaxDivergence()
    rb_launch_s = t["solve_ms"] / 1e3 / t["rbgs_launches"]

    # --- end to end through the C ABI with host buffers ---------------------
    try:
        import torch
        pin = torch.cuda.is_available()
    except ImportError:
        pin = False
    host, back = [], []
    for a in (u, v, w):
        if pin:
            tt = torch.from_numpy(a).pin_memory()
            host.append((tt, tt.data_ptr(), a.size))
            bb = torch.empty(a.size, dtype=torch.float64).pin_memory()
            back.append((bb, bb.data_ptr(), a.size))
        else:
            bb = a.copy()
            host.append((a, a.ctypes.data, a.size))
            back.append((bb, bb.ctypes.data, a.size))
    lib = L.lib()
    out = C.c_double()
    e2e_steps = max(3, args.steps // 2)

    def e2e_step():
        # The drop-in's Mesh.Data mirror: push the caller's fields, Step,
        # pull the fields back, and read the step's MaxDivergence.
        for fid, (_, ptr, n) in zip((1, 2, 3), host):
            e._check(lib.af_field_upload(e._h, fid, ptr, n))
        e._check(lib.af_step(e._h, 1))
        e._check(lib.af_max_divergence(e._h, C.byref(out)))
        for fid, (_, ptr, n) in zip((1, 2, 3), back):
            e._check(lib.af_field_download(e._h, fid, ptr, n))

    e2e_step()  # warm-up (graph rebuild without event nodes)
    dist.barrier()
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        e2e_step()
    e2e_s = dist.max(time.perf_counter() - t0)
    e2e_val = cells * e2e_steps * world / e2e_s
    h2d = 8 * (u.size + v.size + w.size)
    e.Close()

    # --- roofline of the dominant kernel (one red-black colour sweep) --------
    peak, peak_kind = measured_peaks()
    alg_bytes = 1.5 * 8 * cells  # 3b per cell per red+black pair, half per colour launch
    achieved = alg_bytes / rb_launch_s / 1e9
    traffic = profiled_traffic("rbgs_fp64_256")
    fma_rate = C.c_double()
    lib.af_device_fp64_rate(local, C.byref(fma_rate))
    fp64_inst = 6 * cells / 2  # per update: 5 adds and 1 subtract; the exact /6 runs on the integer pipe
    fp64_ach = fp64_inst / rb_launch_s

    # --- mixed precision, at 1e-10 and at the plain form's own max|div| ------
    mixed = {}
    for label, tol in (("mixed", 1e-10), ("mixed_same_div_tol", max(md_plain, 1e-10))):
        em, _ = new_engine(L.AF_PRECISION_MIXED, local, rank, tol)
        tm = device_timed(em, args.steps, args.warmup, dist)
        mv = cells * args.steps * world / tm["dev_s"]
        # Both projections of a step counted as the last one (passes and V-cycles).
        mb = mixed_bytes_per_cell_step(statistics.mean(tm["passes"]), statistics.mean(tm["vcycles"]))
        if label == "mixed":
            mixed_fields, mixed_md = velocity_host(em), em.MaxDivergence()
        mixed[label] = {"value": mv, "unit": UNIT, "ms_per_step": tm["dev_s"] * 1e3 / args.steps,
                        "div_tol": tol, "max_divergence_after": em.MaxDivergence(),
                        "refinement_passes_last_projection": tm["passes"],
                        "vcycles_last_projection": tm["vcycles"],
                        "stages_ms_per_step": {"projections": tm["solve_ms"], "sweeps": tm["sweep_ms"]},
                        "speedup_vs_plain": mv / value,
                        "roofline": {"bound": "hbm", "scope": "whole step", "algorithmic_bytes_per_cell_step": mb,
                                     "achieved": mv / world * mb / 1e9, "peak": peak, "unit": "GB/s",
                                     "frac": mv / world * mb / 1e9 / peak, "peak_source": f"{peak_kind} hbm_gbs"},
                        "dtype": "f32 sweeps and inner multigrid, f64 state/residual/accumulator"}
        em.Close()

    # --- FP64 with the multigrid projection option (exact projection) --------
    ef, _ = new_engine(L.AF_PRECISION_FP64, local, rank)
    ef.EnableMultigridSolver(1e-12)
    tf = device_timed(ef, args.steps, args.warmup, dist)
    fv = cells * args.steps * world / tf["dev_s"]
    mixed["fp64_multigrid"] = {"value": fv, "unit": UNIT, "ms_per_step": tf["dev_s"] * 1e3 / args.steps,
                               "div_tol": 1e-12, "max_divergence_after": ef.MaxDivergence(),
                               "refinement_passes_last_projection": tf["passes"],
                               "stages_ms_per_step": {"projections": tf["solve_ms"], "sweeps": tf["sweep_ms"]},
                               "speedup_vs_plain": fv / value,
                               "dtype": "f64 sweeps (bit-identical to the CPU path); projection: f64 refinement "
                                        "around f32 multigrid (EnableMultigridSolver)"}
    mixed["mixed"]["error_vs_fp64"] = error_vs_fp64(mixed_fields, ef, mixed_md, args.warmup + args.steps)
    del mixed_fields
    ef.Close()

    extra = {}
    if "c3" in args.legs:
        extra["mixed_512"] = bench_mixed_512(args, dist, local, rank)
    if "c4" in args.legs:
        extra["batched"] = bench_batched(args, dist, local)
    if "c5" in args.legs and world == 1:
        extra["served"] = bench_served(args, local)

    dist.close()
    if rank != 0:
        return 0
    line = common_fields(args, world)
    line.update({
        "value": value, "ms_per_step": t["dev_s"] * 1e3 / args.steps, "wall_ms_per_step": t["wall_s"] * 1e3 / args.steps,
        "gpu_launches": t["launches"] * args.steps,
        "e2e": {"value": e2e_val, "unit": UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": h2d + 8,
                "steps": e2e_steps, "host_memory": "pinned" if pin else "pageable",
                "per_step": "upload U, V, W; Step; MaxDivergence; download U, V, W (the Mesh.Data mirror)"},
        "roofline": {"bound": "hbm", "kernel": "k_rbgs_fp64 (one colour sweep)", "achieved": achieved,
                     "peak": peak, "unit": "GB/s", "frac": achieved / peak, "peak_source": f"{peak_kind} hbm_gbs",
                     "traffic": traffic, "launch_us": rb_launch_s * 1e6,
                     "algorithmic_bytes_per_launch": alg_bytes,
                     "fp64_pipe": {"achieved": fp64_ach, "peak": fma_rate.value, "unit": "FP64 inst/s",
                                   "frac": fp64_ach / fma_rate.value if fma_rate.value else None,
                                   "inst_per_update": 6}},
        "stages_ms_per_step": {"rbgs": t["solve_ms"], "sweeps": t["sweep_ms"], "step": t["dev_s"] * 1e3 / args.steps},
        "max_divergence_after": md_plain,
        "clocks": t["clocks"],
        **mixed,
        **extra,
    })
    if world == 1 and not args.no_cpu_baseline:
        threads = cpu_threads()
        sec = run_oracle_steps(0, 1, threads)
        line["cpu_baseline"] = {"value": cells / sec, "unit": UNIT, "cores": threads, "kind": "port",
                                "sample": f"1 Step of the {N}^3 workload on the CPU oracle (C restatement of "
                                          f"the Go path), {threads} worker threads, {sec:.1f} s"}
    print(json.dumps(line), flush=True)
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--legs", default="c3,c4,c5", help="extra measurements: c3 (512^3 mixed), c4 (batched), "
                                                       "c5 (served)")
    ap.add_argument("--serve-seconds", type=float, default=60.0)
    args = ap.parse_args()
    if args.warmup < 3 and args.impl == "ours":
        args.warmup = 3
    if args.impl == "reference":
        return bench_reference(args)
    return bench_ours(args)


if __name__ == "__main__":
    sys.exit(main())
