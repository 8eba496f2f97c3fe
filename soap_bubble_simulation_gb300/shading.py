"""Headless film shading: the bubble fragment shader (bubble.wgsl:486-545) on the GPU.

`BubbleUniform` is the renderer's per-bubble uniform (pipeline.rs:23-111) with the same field
names and defaults; `Camera` is the orbit camera of camera.rs (look-at, right-handed perspective
with depth 0..1); `shade_fragments` colours a batch of fragments; `render_frame` produces one
frame of the headless renderer (render/headless.rs) without a graphics stack: a ray per pixel
finds the bubble's front surface, which is shaded and alpha-blended over the background.
"""
from __future__ import annotations

import ctypes as C
import math
from dataclasses import dataclass

import numpy as np

from . import _native as N
from .interference import generate_interference_lut_array

LUT_ANGLES = 64
LUT_THICKNESSES = 256
BRANCHED_W = 512
BRANCHED_H = 256
HEADLESS_RADIUS = 0.025  # render/headless.rs:334 (5 cm bubble)


class BubbleUniform(C.Structure):
    """pipeline.rs:23-67, field for field (128 bytes)."""

    _fields_ = [(name, C.c_float) for name in (
        "refractive_index", "base_thickness_nm", "time", "interference_intensity", "base_alpha", "edge_alpha",
        "background_r", "background_g", "background_b", "film_time", "swirl_intensity", "drainage_speed",
        "pattern_scale", "position_x", "position_y", "position_z")] + [
        ("edge_smoothing_mode", C.c_uint32), ("branched_flow_enabled", C.c_uint32)] + [
        (name, C.c_float) for name in ("branched_flow_intensity", "branched_flow_scale", "branched_flow_sharpness",
                                       "light_dir_x", "light_dir_y", "light_dir_z")] + [
        ("patch_enabled", C.c_uint32)] + [
        (name, C.c_float) for name in ("patch_center_u", "patch_center_v", "patch_half_size")] + [
        ("padding", C.c_uint32 * 4)]

    @classmethod
    def default(cls) -> "BubbleUniform":
        """BubbleUniform::default() (pipeline.rs:69-111)."""
        u = cls()
        N.call("sbs_bubble_uniform_default", C.cast(C.byref(u), C.c_void_p))
        return u

    def set_time(self, t: float) -> None:
        """HeadlessRenderer::set_time (render/headless.rs:545-548)."""
        self.time = t
        self.film_time = t


assert C.sizeof(BubbleUniform) == 128


@dataclass
class Camera:
    """The orbit camera of camera.rs:20-107 (glam look_at_rh / perspective_rh, wgpu depth 0..1)."""

    aspect: float
    distance: float = 0.2
    yaw: float = 0.0
    pitch: float = 0.3
    fov: float = math.radians(45.0)
    near: float = 0.001
    far: float = 100.0
    target: tuple = (0.0, 0.0, 0.0)

    def position(self) -> np.ndarray:
        x = self.distance * math.cos(self.pitch) * math.sin(self.yaw)
        y = self.distance * math.sin(self.pitch)
        z = self.distance * math.cos(self.pitch) * math.cos(self.yaw)
        return np.asarray(self.target, dtype=np.float64) + np.array([x, y, z])

    def orbit(self, dx: float, dy: float) -> None:
        """Camera::orbit (camera.rs:70-77): yaw and pitch by 0.01 per unit, pitch kept off the poles."""
        self.yaw += dx * 0.01
        self.pitch = min(max(self.pitch + dy * 0.01, -(math.pi / 2 - 0.01)), math.pi / 2 - 0.01)

    def zoom(self, delta: float) -> None:
        """Camera::zoom (camera.rs:80-83): distance scaled by 1 - 0.1 delta, kept in [0.05, 10]."""
        self.distance = min(max(self.distance * (1.0 - delta * 0.1), 0.05), 10.0)

    def set_aspect(self, aspect: float) -> None:
        self.aspect = aspect

    def view_matrix(self) -> np.ndarray:
        """Mat4::look_at_rh(position, target, +y) (camera.rs:91-94), row-major 4 x 4, float64."""
        eye = self.position()
        f = np.asarray(self.target, dtype=np.float64) - eye
        f /= np.linalg.norm(f)
        s = np.cross(f, [0.0, 1.0, 0.0])
        s /= np.linalg.norm(s)
        u = np.cross(s, f)
        view = np.identity(4)
        view[0, :3], view[1, :3], view[2, :3] = s, u, -f
        view[:3, 3] = [-eye @ s, -eye @ u, eye @ f]
        return view

    def projection_matrix(self) -> np.ndarray:
        """Mat4::perspective_rh (depth 0..1) (camera.rs:97-99), row-major 4 x 4, float64."""
        h = math.cos(0.5 * self.fov) / math.sin(0.5 * self.fov)
        r = self.far / (self.near - self.far)
        proj = np.zeros((4, 4))
        proj[0, 0], proj[1, 1], proj[2, 2], proj[3, 2], proj[2, 3] = h / self.aspect, h, r, -1.0, r * self.near
        return proj

    def view_projection_matrix(self) -> np.ndarray:
        return self.projection_matrix() @ self.view_matrix()

    def view_proj(self) -> np.ndarray:
        """Column-major 4 x 4 (as CameraUniform.view_proj), float32, flattened."""
        return self.view_projection_matrix().T.astype(np.float32).ravel()  # row-major of the transpose

    def uniform(self):
        """Camera::uniform (camera.rs:107-114): (view_proj column-major [16] f32, camera_pos [3] f32)."""
        return self.view_proj(), self.position().astype(np.float32)


def _u8(a, shape):
    a = np.ascontiguousarray(a, dtype=np.uint8)
    if a.size != int(np.prod(shape)):
        raise ValueError(f"expected {np.prod(shape)} bytes")
    return a


def default_lut(refractive_index: float = 1.33) -> np.ndarray:
    """The LUT the renderer uploads: generate_interference_lut(n, 1.0), [64][256][4] RGBA8."""
    return generate_interference_lut_array(refractive_index, 1.0)


def shade_fragments(uniform: BubbleUniform, camera_pos, lut, normals, world_pos, branched=None) -> np.ndarray:
    """fs_main for n fragments (normals, world positions [n][3]) -> straight-alpha RGBA [n][4]."""
    nn = np.ascontiguousarray(normals, dtype=np.float32).reshape(-1, 3)
    wp = np.ascontiguousarray(world_pos, dtype=np.float32).reshape(-1, 3)
    if nn.shape != wp.shape:
        raise ValueError("normals and world_pos must have the same shape")
    cam = np.ascontiguousarray(camera_pos, dtype=np.float32).reshape(3)
    L = _u8(lut, (LUT_ANGLES, LUT_THICKNESSES, 4))
    B = None if branched is None else np.ascontiguousarray(branched, dtype=np.uint32).reshape(BRANCHED_H, BRANCHED_W)
    out = np.empty((nn.shape[0], 4), dtype=np.float32)
    N.call("sbs_shade_fragments", C.cast(C.byref(uniform), C.c_void_p), N.ptr(cam), N.ptr(L), N.ptr(B),
           nn.shape[0], N.ptr(nn), N.ptr(wp), N.ptr(out), N.MEM_HOST, None)
    return out


def render_frame(uniform: BubbleUniform, camera: Camera, width: int, height: int, lut=None, branched=None,
                 radius: float = HEADLESS_RADIUS, linear: bool = False):
    """One headless frame: RGBA8 sRGB bytes [height][width][4] (HeadlessRenderer::render_to_buffer
    without the row padding), or linear RGBA f32 with linear=True."""
    vp = camera.view_proj()
    cam = camera.position().astype(np.float32)
    L = _u8(default_lut(uniform.refractive_index) if lut is None else lut, (LUT_ANGLES, LUT_THICKNESSES, 4))
    B = None if branched is None else np.ascontiguousarray(branched, dtype=np.uint32).reshape(BRANCHED_H, BRANCHED_W)
    rgba8 = None if linear else np.empty((height, width, 4), dtype=np.uint8)
    lin = np.empty((height, width, 4), dtype=np.float32) if linear else None
    N.call("sbs_shade_frame", C.cast(C.byref(uniform), C.c_void_p), N.ptr(vp), N.ptr(cam), float(radius), N.ptr(L),
           N.ptr(B), int(width), int(height), N.ptr(rgba8), N.ptr(lin), N.MEM_HOST, None)
    return lin if linear else rgba8
