import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300); runs the CUDA path through the C ABI")
    config.addinivalue_line("markers", "slow: full-size case (seconds to minutes)")


import pytest as _pytest  # noqa: E402


@_pytest.fixture(autouse=True)
def _no_out_of_buffer_accesses(request):
    """Under the bounds-checking debug library (AEROFLUX_DEBUG_BOUNDS=1),
    every GPU test must leave no out-of-buffer access on record."""
    yield
    if os.environ.get("AEROFLUX_DEBUG_BOUNDS") == "1" and request.node.get_closest_marker("gpu"):
        from aeroflux_gb300 import _lib
        enabled, first, n = _lib.debug_bounds(reset=True)
        assert enabled, "AEROFLUX_DEBUG_BOUNDS=1 but the product library is loaded"
        assert n == 0, (f"{n} out-of-buffer accesses; first: kernel {first >> 56}, slot {(first >> 40) & 0xFFFF}, "
                        f"offset {first & 0xFFFFFFFFFF}")
