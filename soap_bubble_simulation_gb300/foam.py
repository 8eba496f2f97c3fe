"""Batched foam drainage: many bubbles with uneven grids advanced by one persistent GPU launch.

Each bubble has its own GPUDrainageSimulator-semantics grid (drainage.wgsl physics, resolution x
2 resolution cells, its own radius). The reference's foam bubbles carry a single scalar thickness
(foam.rs:44); this module gives every bubble a full film instead.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _native as N
from .drainage import DrainageParams


class FoamDrainage:
    def __init__(self, resolution, radius_m, params: DrainageParams | None = None):
        res = np.ascontiguousarray(resolution, dtype=np.uint32)
        rad = np.ascontiguousarray(radius_m, dtype=np.float32)
        if res.size != rad.size:
            raise ValueError("resolution and radius differ in length")
        self.resolution = res.copy()
        self._h = C.c_void_p()
        p = (params or DrainageParams()).to_c()
        N.call("sbs_foam_create", int(res.size), N.ptr(res), N.ptr(rad), C.byref(p), C.byref(self._h))

    def close(self):
        if self._h:
            N.lib().sbs_foam_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __len__(self):
        return int(self.resolution.size)

    def total_cells(self) -> int:
        out = C.c_uint64()
        N.call("sbs_foam_total_cells", self._h, C.byref(out))
        return out.value

    def _io(self, fn, b, a=None):
        r = int(self.resolution[b])
        if a is None:
            out = np.empty((r, 2 * r), dtype=np.float32)
            N.call(fn, self._h, int(b), N.ptr(out), out.size, N.MEM_HOST)
            return out
        a = np.ascontiguousarray(a, dtype=np.float32)
        if a.shape != (r, 2 * r):
            raise ValueError(f"bubble {b} field must be {r} x {2 * r}")
        N.call(fn, self._h, int(b), N.ptr(a), a.size, N.MEM_HOST)

    def set_thickness(self, b, a):
        self._io("sbs_foam_set_thickness", b, a)

    def thickness(self, b) -> np.ndarray:
        return self._io("sbs_foam_get_thickness", b)

    def set_concentration(self, b, a):
        self._io("sbs_foam_set_concentration", b, a)

    def concentration(self, b) -> np.ndarray:
        return self._io("sbs_foam_get_concentration", b)

    def run(self, steps: int):
        N.call("sbs_foam_run", self._h, int(steps))

    def set_tiles(self, steps_per_phase: int, strip_rows: int):
        N.call("sbs_foam_set_tiles", self._h, int(steps_per_phase), int(strip_rows))

    def autotune(self, trial_steps: int = 8) -> tuple[int, int]:
        k, rb = C.c_uint32(), C.c_uint32()
        N.call("sbs_foam_autotune", self._h, int(trial_steps), C.byref(k), C.byref(rb))
        return k.value, rb.value

    def stream(self) -> int:
        out = C.c_void_p()
        N.call("sbs_foam_stream", self._h, C.byref(out))
        return out.value or 0
