"""Builds libaeroflux_cuda.so (the C-ABI engine) in-tree with nvcc for sm_103a.

Each translation unit compiles in parallel to an object under
aeroflux_gb300/_build/, then one nvcc link produces
aeroflux_gb300/libaeroflux_cuda.so.  The library links the CUDA runtime
statically and has no dependency on PyTorch.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libaeroflux_cuda.so")
# The bounds-checking debug build: every kernel load and store checked
# against its buffer (csrc/af_debug.cuh), same ABI, separate objects.
BUILD_DEBUG = os.path.join(HERE, "_build_debug")
LIB_DEBUG = os.path.join(HERE, "libaeroflux_cuda_debug.so")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-ffp-contract=off,-fno-fast-math",
          "-I", INCLUDE, "--expt-relaxed-constexpr"]
# Per-unit flags.  The FP64 plain form and the engine's host arithmetic must
# never contract a*b+c: --fmad=false on top of the explicit intrinsics.
UNITS = {
    "af_engine.cu": ["--fmad=false"],
    "af_fp64.cu": ["--fmad=false"],
    "af_batch.cu": [],
    "af_workload.cu": [],
    "af_serve.cu": [],
}


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libaeroflux_cuda")


def _deps() -> list[str]:
    out = [os.path.join(CSRC, f) for f in os.listdir(CSRC)]
    out += [os.path.join(INCLUDE, f) for f in os.listdir(INCLUDE)]
    return out


def up_to_date(lib: str = LIB) -> bool:
    if not os.path.exists(lib):
        return False
    t = os.path.getmtime(lib)
    return all(os.path.getmtime(p) <= t for p in _deps())


def _compile(unit: str, flags: list[str], verbose: bool, debug_bounds: bool = False) -> str:
    src = os.path.join(CSRC, unit)
    obj = os.path.join(BUILD_DEBUG if debug_bounds else BUILD, unit.replace(".cu", ".o"))
    cmd = [nvcc(), *ARCH, *COMMON, *flags, "-c", src, "-o", obj]
    if debug_bounds:
        cmd.insert(1, "-DAEROFLUX_DEBUG_BOUNDS=1")
    if verbose:
        cmd.insert(1, "-Xptxas=-v")
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed on {unit}:\n{r.stdout}\n{r.stderr}")
    if verbose:
        sys.stderr.write(r.stderr)
    return obj


def build(force: bool = False, verbose: bool = False, debug_bounds: bool = False) -> str:
    """Compile every CUDA unit for sm_103a and link the shared library
    (debug_bounds: the bounds-checking debug library instead)."""
    lib = LIB_DEBUG if debug_bounds else LIB
    if not force and up_to_date(lib):
        return lib
    os.makedirs(BUILD_DEBUG if debug_bounds else BUILD, exist_ok=True)
    with cf.ThreadPoolExecutor(max_workers=len(UNITS)) as ex:
        objs = list(ex.map(lambda kv: _compile(kv[0], kv[1], verbose, debug_bounds), UNITS.items()))
    tmp = lib + ".tmp"
    cmd = [nvcc(), *ARCH, "-shared", "-o", tmp, *objs, "-Xcompiler", "-fPIC"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, lib)
    return lib


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv, debug_bounds="--debug-bounds" in sys.argv))
