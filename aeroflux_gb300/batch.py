"""Batched form over the C ABI (af_batch_*): many mixed-precision grids of
uneven sizes stepping together, one persistent launch per stage, one CUDA
graph per step.  Slots can be assigned and released between steps."""
from __future__ import annotations

import ctypes as C
import json

import numpy as np

from . import _lib as L
from .engine import FIELD_IDS, AerofluxError, Config, Field


class Batch:
    def __init__(self, capacity: int, pool_bytes: int = 0, device: int = 0):
        h = C.c_void_p()
        buf = C.create_string_buffer(512)
        rc = L.lib().af_batch_create(capacity, pool_bytes, device, C.byref(h), buf, 512)
        if rc != L.AF_OK:
            raise AerofluxError(buf.value.decode(), rc)
        self._h = h
        self.capacity = capacity

    def _check(self, rc: int) -> None:
        if rc != L.AF_OK:
            raise AerofluxError((L.lib().af_batch_last_error(self._h) or b"").decode(), rc)

    @staticmethod
    def slot_bytes(cfg: Config) -> int:
        n = C.c_int64()
        rc = L.lib().af_batch_slot_bytes(C.byref(cfg.to_c()), C.byref(n))
        if rc != L.AF_OK:
            raise AerofluxError("aeroflux: invalid configuration", rc)
        return n.value

    def assign(self, cfg: Config) -> int:
        s = C.c_int64()
        self._check(L.lib().af_batch_assign(self._h, C.byref(cfg.to_c()), C.byref(s)))
        return s.value

    def release(self, slot: int) -> None:
        self._check(L.lib().af_batch_release(self._h, slot))

    def set_active(self, slot: int, active: bool) -> None:
        self._check(L.lib().af_batch_set_active(self._h, slot, int(active)))

    def config(self, slot: int) -> Config:
        c = L.AfConfig()
        self._check(L.lib().af_batch_get_config(self._h, slot, C.byref(c)))
        return Config.from_c(c)

    def field(self, slot: int, name: str) -> Field:
        d = L.AfFieldDesc()
        self._check(L.lib().af_batch_field_info(self._h, slot, FIELD_IDS[name], C.byref(d)))
        return Field(d.off, d.nx, d.ny, d.nz, d.sy, d.sz, d.count, name)

    def upload(self, slot: int, name: str, arr: np.ndarray) -> None:
        a = np.ascontiguousarray(arr, dtype=np.float64)
        self._check(L.lib().af_batch_field_upload(self._h, slot, FIELD_IDS[name], a.ctypes.data, a.size))

    def upload_ptr(self, slot: int, name: str, ptr: int, count: int) -> None:
        self._check(L.lib().af_batch_field_upload(self._h, slot, FIELD_IDS[name], ptr, count))

    def download(self, slot: int, name: str, out: np.ndarray | None = None) -> np.ndarray:
        if out is None:
            out = np.empty(self.field(slot, name).Count)
        self._check(L.lib().af_batch_field_download(self._h, slot, FIELD_IDS[name], out.ctypes.data, out.size))
        return out

    def seed(self, slot: int, amp: float = 1.0, noise: float = 0.01, seed: int = 42, stream: int = 0) -> None:
        """Device-side Taylor-Green + PCG32 initial field (then apply the BC)."""
        self._check(L.lib().af_batch_seed(self._h, slot, amp, noise, seed, stream))

    def apply_velocity_bc(self) -> None:
        self._check(L.lib().af_batch_apply_velocity_bc(self._h))

    def step(self, n: int = 1) -> None:
        self._check(L.lib().af_batch_step(self._h, n))

    def status(self, slot: int) -> tuple[bool, str]:
        f = C.c_int32()
        buf = C.create_string_buffer(512)
        self._check(L.lib().af_batch_slot_status(self._h, slot, C.byref(f), buf, 512))
        return bool(f.value), buf.value.decode()

    def max_divergence(self, slot: int) -> float:
        out = C.c_double()
        self._check(L.lib().af_batch_max_divergence(self._h, slot, C.byref(out)))
        return out.value

    def projection_stats(self, slot: int) -> tuple[int, float]:
        p, d = C.c_int64(), C.c_double()
        self._check(L.lib().af_batch_projection_stats(self._h, slot, C.byref(p), C.byref(d)))
        return p.value, d.value

    def tune(self, reps: int = 5) -> dict:
        buf = C.create_string_buffer(1 << 16)
        self._check(L.lib().af_batch_tune(self._h, reps, buf, 1 << 16))
        return json.loads(buf.value.decode())

    def profile(self, on: bool = True) -> None:
        self._check(L.lib().af_batch_profile(self._h, int(on)))

    def last_step_profile(self) -> L.AfStepProfile:
        p = L.AfStepProfile()
        self._check(L.lib().af_batch_last_step_profile(self._h, C.byref(p)))
        return p

    def close(self) -> None:
        if self._h:
            L.lib().af_batch_destroy(self._h)
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
