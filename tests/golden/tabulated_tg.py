"""A host-reproducible Taylor-Green + PCG32 initial field for large fixtures.

TEST INFRASTRUCTURE.  The product's generator (af_seed_taylor_green) calls
libm sin/cos, whose last bits may differ between the x86 host that made a
fixture and the Arm host that checks it.  On a cube of extent N every face
coordinate is a multiple of H/2 = 1/(2N), so the vortex needs only
sin(2*pi*m/(2N)) and cos(2*pi*m/(2N)) for m = 0..2N: those tables are stored
with the fixture, and everything else is IEEE arithmetic that numpy evaluates
without contraction:

    u = ((amp * sin X) * cos Y) * cos Z + noise * (2 * uniform - 1)
    v = ((-amp * cos X) * sin Y) * cos Z + noise * (2 * uniform - 1)
    w = 0.0 + noise * (2 * uniform - 1)

written over seedVortex's index ranges (engine_test.go:313-333) in field
order U, V, W and z, y, x loop order, each uniform a 53-bit double from two
PCG32 outputs (O'Neill 2014, XSH-RR 64/32, pcg32_srandom_r seeding) -- the
same sequence as the product's generator, produced here with vectorised
jump-ahead (F. Brown, "Random number generation with arbitrary strides",
1994) instead of a Python loop.
"""
from __future__ import annotations

import numpy as np

MULT = np.uint64(6364136223846793005)


def trig_tables(n: int) -> tuple[np.ndarray, np.ndarray]:
    """sin and cos of 2*pi*m/(2n), m = 0..2n (the values the fixture stores)."""
    m = np.arange(2 * n + 1, dtype=np.float64)
    a = 2.0 * np.pi * (m / (2.0 * n))
    return np.sin(a), np.cos(a)


def _pcg_states(seed: int, stream: int, count: int, chunk: int = 1 << 22):
    """Yields arrays of consecutive PCG32 states (the `old` of each output)."""
    M = (1 << 64) - 1
    inc = ((stream << 1) | 1) & M
    st = inc  # 0 * MULT + inc
    st = (st + seed) & M
    st = (st * int(MULT) + inc) & M
    inc64 = np.uint64(inc)
    # States 0 .. chunk-1 by doubling: S[j + k] = A_k S[j] + C_k.
    base = np.array([st], dtype=np.uint64)
    a, c = int(MULT), inc
    with np.errstate(over="ignore"):
        while base.size < chunk:
            nxt = base * np.uint64(a) + np.uint64(c)
            base = np.concatenate([base, nxt])
            a, c = (a * a) & M, (a * c + c) & M
        base = base[:chunk]
        # A_chunk, C_chunk for stepping a whole chunk.
        ak, ck, k, aa, cc = 1, 0, chunk, int(MULT), inc
        while k:
            if k & 1:
                ak, ck = (ak * aa) & M, (ck * aa + cc) & M
            aa, cc = (aa * aa) & M, (aa * cc + cc) & M
            k >>= 1
        done = 0
        cur = base
        while done < count:
            take = min(chunk, count - done)
            yield cur[:take]
            done += take
            cur = cur * np.uint64(ak) + np.uint64(ck)
    del inc64


def _outputs(old: np.ndarray) -> np.ndarray:
    xs = (((old >> np.uint64(18)) ^ old) >> np.uint64(27)) & np.uint64(0xFFFFFFFF)
    rot = old >> np.uint64(59)
    out = (xs >> rot) | (xs << ((np.uint64(32) - rot) & np.uint64(31)))
    return out & np.uint64(0xFFFFFFFF)


def uniforms(seed: int, stream: int, n: int) -> np.ndarray:
    """n draws of the 53-bit uniform in [0, 1) (two outputs each)."""
    parts = []
    for old in _pcg_states(seed, stream, 2 * n):
        parts.append(_outputs(old))
    o = np.concatenate(parts) if parts else np.zeros(0, dtype=np.uint64)
    a = (o[0::2] >> np.uint64(5)).astype(np.float64)
    b = (o[1::2] >> np.uint64(6)).astype(np.float64)
    return (a * 67108864.0 + b) * (1.0 / 9007199254740992.0)


def tabulated_taylor_green(n: int, ghost: int, sin_t: np.ndarray, cos_t: np.ndarray, amp: float, noise: float,
                           seed: int, stream: int = 0):
    """Padded host arrays (u, v, w) of an n^3 grid with H = 1/n."""
    g = ghost
    cx = cy = cz = n + 2 * g
    uni = uniforms(seed, stream, n * n * (n + 1) * 3)
    jit = noise * (2.0 * uni - 1.0)
    nu = n * n * (n + 1)
    ju, jv, jw = jit[:nu], jit[nu:2 * nu], jit[2 * nu:]
    i = np.arange(n + 1)
    # Face coordinates in units of H/2: integer positions 2i, half positions 2i+1.
    S_int, C_int, C_half, S_half = sin_t[2 * i], cos_t[2 * i], cos_t[2 * i[:n] + 1], sin_t[2 * i[:n] + 1]
    u = np.zeros((cz, cy, cx + 1))
    # U: x in [g, g+n], y, z in [g, g+n): X = (x-g) H, Y = (y-g+1/2) H, Z = (z-g+1/2) H.
    tu = ((amp * S_int[None, None, :]) * C_half[None, :, None]) * C_half[:, None, None]
    u[g:g + n, g:g + n, g:g + n + 1] = tu + ju.reshape(n, n, n + 1)
    v = np.zeros((cz, cy + 1, cx))
    tv = ((-amp * C_half[None, None, :]) * S_int[None, :, None]) * C_half[:, None, None]
    v[g:g + n, g:g + n + 1, g:g + n] = tv + jv.reshape(n, n + 1, n)
    w = np.zeros((cz + 1, cy, cx))
    w[g:g + n + 1, g:g + n, g:g + n] = 0.0 + jw.reshape(n + 1, n, n)
    return u.ravel(), v.ravel(), w.ravel()
