"""Caustic intensity map over the film thickness (caustics_compute.wgsl, caustics.rs).

`CausticParams` is the renderer's uniform (caustics.rs:17-76) with the same field names and
defaults; `caustic_map` runs the compute pass on a host field; `GPUDrainageSimulator.caustic_map`
runs it on the simulator's own device field without a copy.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _native as N


class CausticParams(C.Structure):
    """caustics.rs:17-52, field for field (64 bytes)."""

    _fields_ = [("grid_width", C.c_uint32), ("grid_height", C.c_uint32)] + [
        (name, C.c_float) for name in (
            "refractive_index", "film_thickness_scale", "light_dir_x", "light_dir_y", "light_dir_z",
            "light_intensity", "focal_length", "caustic_intensity", "caustic_sharpness", "branch_threshold",
            "ground_y", "bubble_radius", "time")] + [("padding", C.c_uint32)]

    @classmethod
    def default(cls, grid_width: int | None = None, grid_height: int | None = None) -> "CausticParams":
        """CausticParams::default() (caustics.rs:54-76), optionally for another grid."""
        p = cls()
        N.call("sbs_caustic_params_default", C.cast(C.byref(p), C.c_void_p))
        if grid_width is not None:
            p.grid_width = int(grid_width)
        if grid_height is not None:
            p.grid_height = int(grid_height)
        return p


assert C.sizeof(CausticParams) == 64


def caustic_map(params: CausticParams, thickness) -> np.ndarray:
    """The caustic compute pass over a [grid_height][grid_width] f32 thickness field."""
    h = np.ascontiguousarray(thickness, dtype=np.float32)
    if h.shape != (params.grid_height, params.grid_width):
        raise ValueError("thickness must be grid_height x grid_width")
    out = np.empty_like(h)
    N.call("sbs_caustics", C.cast(C.byref(params), C.c_void_p), N.ptr(h), h.shape[1], N.ptr(out), N.MEM_HOST, None)
    return out
