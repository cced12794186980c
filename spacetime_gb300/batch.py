"""Batched stepping of many condensates (gpe_batch_*): one cooperative persistent
kernel advances every member, and an n-step run can be recorded into one CUDA
graph and replayed.  The members are ordinary Steppers; after a batched call
each of them is where gpe_step(n) would have left it."""
from __future__ import annotations

import ctypes as C
import json

from . import capi


class Batch:
    def __init__(self, steppers):
        self.lib = capi.load_library()
        self.members = list(steppers)
        arr = (C.c_void_p * len(self.members))(*[s._h.value for s in self.members])
        self._b = C.c_void_p()
        capi.check(self.lib.gpe_batch_create(arr, len(self.members), C.byref(self._b)), "gpe_batch_create")
        self.stream = None

    def close(self):
        if getattr(self, "_b", None):
            self.lib.gpe_batch_destroy(self._b)
            self._b = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def step(self, n: int):
        capi.check(self.lib.gpe_batch_step(self._b, n, self.stream), "gpe_batch_step")

    def capture(self, n: int, stream):
        """Record an n-step run into a CUDA graph on `stream` (a non-default stream handle)."""
        capi.check(self.lib.gpe_batch_capture(self._b, n, stream), "gpe_batch_capture")

    def replay(self, stream=None):
        capi.check(self.lib.gpe_batch_replay(self._b, stream if stream is not None else self.stream), "gpe_batch_replay")

    def set_tuning(self, key: int, value: int):
        capi.check(self.lib.gpe_batch_set_tuning(self._b, key, value), "gpe_batch_set_tuning")

    def get_tuning(self, key: int) -> int:
        v = C.c_int32()
        capi.check(self.lib.gpe_batch_get_tuning(self._b, key, C.byref(v)), "gpe_batch_get_tuning")
        return v.value

    def autotune(self, steps: int = 4) -> list:
        buf = C.create_string_buffer(1 << 16)
        capi.check(self.lib.gpe_batch_autotune(self._b, steps, buf, len(buf), self.stream), "gpe_batch_autotune")
        return json.loads(buf.value.decode() or "[]")

    @property
    def sites(self) -> int:
        return int(self.lib.gpe_batch_sites(self._b))

    @property
    def launches(self) -> int:
        return int(self.lib.gpe_batch_launch_count(self._b))
