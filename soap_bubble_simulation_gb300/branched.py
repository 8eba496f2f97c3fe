"""Branched flow of light through the film (branched_flow.rs, branched_flow_compute.wgsl).

`BranchedFlowParams` is the renderer's uniform (branched_flow.rs:43-134) with the same field names
and defaults; `generate_scatterers` is branched_flow.rs:164-226 (host); `BranchedFlowSimulator`
keeps the u32 texture and advances it like the reference's `step` (fade, then trace). The texture
is what the bubble shader samples (`shade_fragments(..., branched=texture)`).
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _native as N

MAX_SCATTERERS = 2048


class BranchedFlowParams(C.Structure):
    """branched_flow.rs:43-94, field for field (112 bytes)."""

    _fields_ = [("entry_point", C.c_float * 3), ("beam_dir", C.c_float * 3), ("num_rays", C.c_uint32),
                ("ray_steps", C.c_uint32)] + [
        (n, C.c_float) for n in ("step_size", "bend_strength", "spread_angle", "intensity_falloff")] + [
        ("tex_width", C.c_uint32), ("tex_height", C.c_uint32)] + [
        (n, C.c_float) for n in ("time", "thickness_scale", "base_thickness_nm", "swirl_intensity", "drainage_speed",
                                 "pattern_scale")] + [
        ("num_scatterers", C.c_uint32)] + [
        (n, C.c_float) for n in ("scatterer_strength", "scatterer_radius", "particle_weight")] + [
        ("patch_enabled", C.c_uint32)] + [(n, C.c_float) for n in ("patch_center_u", "patch_center_v",
                                                                    "patch_half_size")]

    @classmethod
    def default(cls) -> "BranchedFlowParams":
        """BranchedFlowParams::default() (branched_flow.rs:96-134)."""
        p = cls()
        N.call("sbs_branched_params_default", C.cast(C.byref(p), C.c_void_p))
        return p


assert C.sizeof(BranchedFlowParams) == 112


def generate_scatterers(params: BranchedFlowParams, num: int | None = None, time: float = 0.0) -> np.ndarray:
    """[num][4] float32 (pos_u, pos_v, strength, inv_sigma_sq): Halton positions with time jitter,
    confined to the patch when params.patch_enabled."""
    n = params.num_scatterers if num is None else int(num)
    out = np.empty((n, 4), dtype=np.float32)
    N.call("sbs_branched_scatterers", C.cast(C.byref(params), C.c_void_p), n, float(time), N.ptr(out))
    return out


def branched_flow_step(params: BranchedFlowParams, thickness, scatterers, texture, fade: bool = True) -> np.ndarray:
    """One fade + trace step on host arrays; returns the new [tex_height][tex_width] u32 texture."""
    th = np.ascontiguousarray(thickness, dtype=np.float32)
    sc = np.ascontiguousarray(scatterers, dtype=np.float32).reshape(-1, 4)
    if sc.shape[0] < min(params.num_scatterers, MAX_SCATTERERS):
        raise ValueError("fewer scatterers than params.num_scatterers")
    tex = np.array(texture, dtype=np.uint32, copy=True).reshape(params.tex_height, params.tex_width)
    N.call("sbs_branched_flow", C.cast(C.byref(params), C.c_void_p), N.ptr(th), th.shape[1], th.shape[0],
           th.shape[1], N.ptr(sc), N.ptr(tex), 1 if fade else 0, N.MEM_HOST, None)
    return tex


class BranchedFlowSimulator:
    """BranchedFlowSimulator (branched_flow.rs:243-601) over a host texture: step() fades the
    texture and traces params.num_rays rays through the given thickness field."""

    def __init__(self, params: BranchedFlowParams | None = None):
        self.params = params if params is not None else BranchedFlowParams.default()
        self.texture = np.zeros((self.params.tex_height, self.params.tex_width), dtype=np.uint32)
        self.scatterers = generate_scatterers(self.params, time=0.0)

    def texture_size(self) -> tuple[int, int]:
        return self.params.tex_width, self.params.tex_height

    def step(self, thickness, time: float) -> np.ndarray:
        self.params.time = time
        self.texture = branched_flow_step(self.params, thickness, self.scatterers, self.texture, fade=True)
        return self.texture
