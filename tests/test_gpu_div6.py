"""Exact binary64 arithmetic on the integer pipe.

The red-black update divides by 6 without the IEEE division sequence: an
integer-pipe form (significand times the 2^65/3 magic, remainder decides the
rounding) in the kernel, and an FMA-remainder form kept as a cross-check.
Both must equal IEEE x/6 for every binary64 input, specials included; the
device self-test compares them on random bit patterns covering every
exponent."""
import ctypes as C

import pytest

from aeroflux_gb300 import _lib as L

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("seed", [1, 2, 0xDEADBEEF, 2 ** 63 + 12345])
def test_exact_div6_matches_ieee_division(seed):
    bad = C.c_int64(-1)
    assert L.lib().af_selftest_div6(0, 100_000_000, seed, C.byref(bad)) == L.AF_OK
    assert bad.value == 0


@pytest.mark.parametrize("seed", [3, 4, 0xC0FFEE, 2 ** 62 + 7])
def test_integer_pipe_add_matches_native(seed):
    bad = C.c_int64(-1)
    assert L.lib().af_selftest_dadd(0, 100_000_000, seed, C.byref(bad)) == L.AF_OK
    assert bad.value == 0
