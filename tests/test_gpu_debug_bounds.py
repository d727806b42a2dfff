"""The kernels stay inside their buffers: the small parity, mixed-precision
and batched cases run under the bounds-checking debug library.

libaeroflux_cuda_debug.so is the same engine built with
AEROFLUX_DEBUG_BOUNDS=1 (aeroflux_gb300/csrc/af_debug.cuh): every device load
and store of every kernel -- the FP64 stages, the binary32 sweeps (row and
TMA-staged, shared-memory tiles included), the multigrid kernels with their
packed 32-bit tile decoding, the one-block tail -- checks the element against
the buffer it addresses.  A violation is recorded, never trapped, and fails
the test that made it (tests/conftest.py).  The cases run in a child process
that loads the debug library, over random ghosts, odd and non-cubic grids,
degenerate axes, narrow tile columns and uneven batches.
"""
import os
import subprocess
import sys

import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SUITES = ["tests/test_gpu_parity.py", "tests/test_gpu_mixed_bits.py", "tests/test_gpu_batch.py",
          "tests/test_gpu_multigrid.py", "tests/test_gpu_maccormack.py"]


def test_small_cases_touch_nothing_outside_their_buffers():
    subprocess.run([sys.executable, "-c", "from aeroflux_gb300 import build as b; b.build(debug_bounds=True)"],
                   cwd=ROOT, check=True)
    env = dict(os.environ, AEROFLUX_DEBUG_BOUNDS="1")
    r = subprocess.run([sys.executable, "-m", "pytest", *SUITES, "-q", "-x", "-m", "gpu and not slow",
                        "-p", "no:cacheprovider"], cwd=ROOT, env=env, capture_output=True, text=True, timeout=1500)
    print(r.stdout[-2000:])
    assert r.returncode == 0, r.stdout[-4000:] + r.stderr[-2000:]
    assert " passed" in r.stdout
