"""Headless film shading on the GPU (sbs_shade_fragments / sbs_shade_frame) against the oracle's
restatement of bubble.wgsl and render/headless.rs.

Bars: fragment colours and alphas within 2e-5 absolute. Everything but the gravity ripple's sin,
the branched-flow atan2 / acos / pow and the sRGB pow is the same FP32 operation sequence on both
sides, and those functions agree to about an ulp; the branched-flow test uses a smooth texture
(a white-noise texture turns an ulp of texture coordinate into 1e-4 of colour).
Frames: each side computes the inverse view-projection on its own (float on the GPU path,
double Gauss-Jordan in the oracle), so rays differ in the last bits: hit points by ~1e-6 of the
radius, which the 24-per-unit noise octaves and the LUT's colour gradient turn into up to ~1e-3
of colour, and at the silhouette a ray can hit on one side and miss on the other. So: at least
97 % of pixels within 1e-4 (linear), sRGB bytes within one step on 99 % of pixels, and at most
0.5 % of pixels (the silhouette) beyond 1e-2.
"""
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def sh(sbs):
    from soap_bubble_simulation_gb300 import shading

    return shading


def sphere_fragments(n, seed, radius=0.025):
    g = np.random.default_rng(seed)
    v = g.normal(size=(n, 3))
    v /= np.linalg.norm(v, axis=1, keepdims=True)
    # interpolated (not unit) normals, as a rasteriser delivers them
    nn = (v * g.uniform(0.97, 1.03, (n, 1))).astype(np.float32)
    return nn, (v * radius).astype(np.float32)


def variants(sh):
    out = []
    for kw in ({}, {"edge_smoothing_mode": 0}, {"edge_smoothing_mode": 2}, {"film_time": 7.5, "time": 7.5},
               {"swirl_intensity": 2.5, "pattern_scale": 1.7, "film_time": 30.0},
               {"base_thickness_nm": 40.0},  # the lower film (x 0.6 at the bottom) below the 30 nm cut
               {"interference_intensity": 1.0, "refractive_index": 1.4}):
        u = sh.BubbleUniform.default()
        for k, v in kw.items():
            setattr(u, k, v)
        out.append(u)
    return out


def test_uniform_default_matches_the_renderer(sh):
    u = sh.BubbleUniform.default()
    assert abs(u.refractive_index - 1.33) < 1e-7 and u.base_thickness_nm == 500.0
    assert u.interference_intensity == 4.0 and u.edge_smoothing_mode == 1 and u.patch_enabled == 1
    assert abs(u.patch_half_size - 0.158) < 1e-7 and u.branched_flow_enabled == 0


def test_fragments_match_oracle(sbs, orc, sh):
    lut = sh.default_lut(1.33)
    nn, wp = sphere_fragments(20000, 1)
    cams = [(0.0, 0.06, 0.19), (0.15, -0.1, 0.05), (0.0, 1.0, 0.0)]
    for k, u in enumerate(variants(sh)):
        cam = cams[k % len(cams)]
        got = sh.shade_fragments(u, cam, lut, nn, wp)
        want = orc.shade_fragments(u, cam, lut, nn, wp)
        d = np.abs(got - want).max()
        assert d <= 2e-5, (k, d)
    # the black-film variant produced black fragments
    u = variants(sh)[5]
    got = sh.shade_fragments(u, cams[0], lut, nn, wp)
    assert np.mean(np.all(np.abs(got[:, :3] - 0.02) < 1e-7, axis=1)) > 0.05


def test_fragments_with_branched_flow(sbs, orc, sh):
    lut = sh.default_lut(1.33)
    g = np.random.default_rng(3)
    yy, xx = np.mgrid[0:sh.BRANCHED_H, 0:sh.BRANCHED_W]
    tex = ((1.2 + np.sin(xx * 2 * np.pi / sh.BRANCHED_W * 3) * np.cos(yy * np.pi / sh.BRANCHED_H * 2)) * 256)
    tex = tex.astype(np.uint32)
    nn, wp = sphere_fragments(20000, 4)
    for patch in (0, 1):
        u = sh.BubbleUniform.default()
        u.branched_flow_enabled = 1
        u.patch_enabled = patch
        u.branched_flow_intensity = 1.3
        u.branched_flow_sharpness = 1.7
        got = sh.shade_fragments(u, (0.0, 0.06, 0.19), lut, nn, wp, branched=tex)
        want = orc.shade_fragments(u, (0.0, 0.06, 0.19), lut, nn, wp, branched=tex)
        assert np.abs(got - want).max() <= 2e-5, patch
        # the texture brightened some fragments beyond the plain film colour
        plain = sh.shade_fragments(sh.BubbleUniform.default(), (0.0, 0.06, 0.19), lut, nn, wp)
        assert (got[:, 0] > plain[:, 0] + 1e-3).mean() > (0.01 if patch else 0.3)


@pytest.mark.parametrize("w,h,yaw,pitch", [(160, 90, 0.0, 0.3), (97, 131, 1.1, -0.4), (64, 64, 2.5, 1.2)])
def test_frame_matches_oracle(sbs, orc, sh, w, h, yaw, pitch):
    lut = sh.default_lut(1.33)
    cam = sh.Camera(aspect=w / h, yaw=yaw, pitch=pitch)
    u = sh.BubbleUniform.default()
    u.set_time(2.0)
    lin = sh.render_frame(u, cam, w, h, lut=lut, linear=True)
    rgba8 = sh.render_frame(u, cam, w, h, lut=lut)
    want8, want_lin = orc.shade_frame(u, cam.view_proj(), cam.position(), sh.HEADLESS_RADIUS, lut, w, h)
    d = np.abs(lin - want_lin).max(axis=-1)
    assert (d <= 1e-4).mean() >= 0.97, (d <= 1e-4).mean()
    assert (d > 1e-2).mean() <= 0.005, (d > 1e-2).mean()
    d8 = np.abs(rgba8.astype(int) - want8.astype(int)).max(axis=-1)
    assert (d8 <= 1).mean() >= 0.99, (d8 <= 1).mean()
    # the bubble's disc: radius tan(asin(R / d)) / tan(fov / 2) of the half height
    bg = np.array([u.background_r, u.background_g, u.background_b])
    hit = np.any(np.abs(lin[..., :3] - bg) > 1e-6, axis=-1)
    r = math.tan(math.asin(0.025 / 0.2)) / math.tan(math.radians(22.5))
    assert abs(hit.mean() - math.pi * r * r / (4 * w / h)) < 0.02


def test_device_memory_frame(sbs, sh):
    import ctypes

    import torch

    N = sbs._native
    lut = torch.from_numpy(sh.default_lut(1.33).copy()).cuda()
    u = sh.BubbleUniform.default()
    cam = sh.Camera(aspect=16 / 9)
    w, h = 320, 180
    out8 = torch.empty((h, w, 4), dtype=torch.uint8, device="cuda")
    vp = cam.view_proj()
    pos = cam.position().astype(np.float32)
    N.call("sbs_shade_frame", ctypes.cast(ctypes.byref(u), ctypes.c_void_p), N.ptr(vp), N.ptr(pos),
           float(sh.HEADLESS_RADIUS), ctypes.c_void_p(lut.data_ptr()), None, w, h,
           ctypes.c_void_p(out8.data_ptr()), None, N.MEM_DEVICE, None)
    torch.cuda.synchronize()
    host = sh.render_frame(u, cam, w, h)
    assert np.array_equal(out8.cpu().numpy(), host)


def test_bad_arguments(sbs, sh):
    u = sh.BubbleUniform.default()
    u.edge_smoothing_mode = 3
    with pytest.raises(sbs.SbsError):
        sh.shade_fragments(u, (0, 0, 1), sh.default_lut(), [(0, 0, 1)], [(0, 0, 0.025)])
    cam = sh.Camera(aspect=1.0)
    with pytest.raises(sbs.SbsError):
        sh.render_frame(sh.BubbleUniform.default(), cam, 8, 8, radius=-1.0)
