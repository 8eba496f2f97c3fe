"""The bubble fragment-shader oracle (bubble.wgsl restated in oracle/shade.cpp), pinned without a
graphics stack: the simplex noise against an independent numpy restatement of the same WGSL (bit
for bit, float32), and closed forms for the terms that do not involve noise: the drainage
profile, the LUT lookup at texel centres, the black-film cut, the three edge-smoothing modes and
the background / blend of a headless frame."""
import math

import numpy as np
import pytest

f32 = np.float32


def np_simplex(v):
    """simplex_noise_3d (bubble.wgsl:113-180) in numpy float32, expression by expression."""
    v = v.astype(f32)
    Cx, Cy = f32(1.0) / f32(6.0), f32(1.0) / f32(3.0)
    s = v[:, 0] * Cy + v[:, 1] * Cy + v[:, 2] * Cy
    i = np.floor(v + s[:, None])
    t = i[:, 0] * Cx + i[:, 1] * Cx + i[:, 2] * Cx
    x0 = v - i + t[:, None]
    g = (x0[:, [0, 1, 2]] >= x0[:, [1, 2, 0]]).astype(f32)  # step(x0.yzx, x0.xyz)
    l = f32(1) - g
    i1 = np.minimum(g, l[:, [2, 0, 1]])
    i2 = np.maximum(g, l[:, [2, 0, 1]])
    x1 = x0 - i1 + Cx
    x2 = x0 - i2 + Cy
    x3 = x0 - f32(0.5)
    i = np.fmod(i, f32(289))

    def permute(x):
        return np.fmod((x * f32(34) + f32(1)) * x, f32(289))

    z4 = np.zeros_like(i[:, 0])
    o4 = np.ones_like(i[:, 0])

    def vec(a, c):
        return np.stack([z4 + 0, i1[:, c], i2[:, c], o4], axis=1) * f32(1)

    p = permute(i[:, 2:3] + vec(0, 2))
    p = permute(p + i[:, 1:2] + vec(0, 1))
    p = permute(p + i[:, 0:1] + vec(0, 0))
    n_ = f32(0.142857142857)
    nsx, nsy, nsz = n_ * f32(2) - f32(0), n_ * f32(0.5) - f32(1), n_ * f32(1) - f32(0)
    j = p - f32(49) * np.floor(p * nsz * nsz)
    x_ = np.floor(j * nsz)
    y_ = np.floor(j - f32(7) * x_)
    x = x_ * nsx + nsy
    y = y_ * nsx + nsy
    h = f32(1) - np.abs(x) - np.abs(y)
    b0 = np.stack([x[:, 0], x[:, 1], y[:, 0], y[:, 1]], axis=1)
    b1 = np.stack([x[:, 2], x[:, 3], y[:, 2], y[:, 3]], axis=1)
    s0 = np.floor(b0) * f32(2) + f32(1)
    s1 = np.floor(b1) * f32(2) + f32(1)
    sh = -(f32(0) >= h).astype(f32)
    a0 = b0[:, [0, 2, 1, 3]] + s0[:, [0, 2, 1, 3]] * sh[:, [0, 0, 1, 1]]
    a1 = b1[:, [0, 2, 1, 3]] + s1[:, [0, 2, 1, 3]] * sh[:, [2, 2, 3, 3]]
    P = [np.stack([a0[:, 0], a0[:, 1], h[:, 0]], 1), np.stack([a0[:, 2], a0[:, 3], h[:, 1]], 1),
         np.stack([a1[:, 0], a1[:, 1], h[:, 2]], 1), np.stack([a1[:, 2], a1[:, 3], h[:, 3]], 1)]

    def dot(a, b):
        return a[:, 0] * b[:, 0] + a[:, 1] * b[:, 1] + a[:, 2] * b[:, 2]

    P = [q * (f32(1.79284291400159) - f32(0.85373472095314) * dot(q, q))[:, None] for q in P]
    X = [x0, x1, x2, x3]
    m = [np.maximum(f32(0.6) - dot(xx, xx), f32(0)) for xx in X]
    m = [mm * mm for mm in m]
    mm = [q * q for q in m]
    d = [dot(P[k], X[k]) for k in range(4)]
    return f32(42) * (mm[0] * d[0] + mm[1] * d[1] + mm[2] * d[2] + mm[3] * d[3])


def test_simplex_matches_independent_numpy_restatement(orc):
    g = np.random.default_rng(0)
    pts = np.concatenate([g.uniform(-40, 40, (4000, 3)), g.uniform(-2, 2, (2000, 3)),
                          np.round(g.uniform(-10, 10, (500, 3)) * 4) / 4]).astype(np.float32)
    want = np_simplex(pts)
    got = np.array([orc.simplex3(*p) for p in pts], dtype=np.float32)
    np.testing.assert_array_equal(got, want)
    assert np.abs(got).max() < 1.05 and abs(float(got.mean())) < 0.05 and got.std() > 0.1


def test_simplex_is_continuous(orc):
    g = np.random.default_rng(1)
    for p in g.uniform(-20, 20, (300, 3)):
        d = g.normal(size=3)
        d *= 1e-4 / np.linalg.norm(d)
        assert abs(orc.simplex3(*p) - orc.simplex3(*(p + d))) < 5e-3


@pytest.fixture(scope="module")
def shading():
    from soap_bubble_simulation_gb300 import shading

    return shading


def _uniform(shading, **kw):
    u = shading.BubbleUniform()
    defaults = dict(refractive_index=1.33, base_thickness_nm=500.0, interference_intensity=4.0, base_alpha=0.3,
                    edge_alpha=0.6, background_r=0.1, background_g=0.1, background_b=0.15, swirl_intensity=1.0,
                    drainage_speed=0.5, pattern_scale=1.0, edge_smoothing_mode=1, branched_flow_intensity=1.0,
                    branched_flow_scale=5.0, branched_flow_sharpness=2.0, light_dir_x=0.577, light_dir_y=0.577,
                    light_dir_z=0.577, patch_enabled=1, patch_center_u=0.5, patch_center_v=0.5,
                    patch_half_size=0.158)
    defaults.update(kw)
    for k, v in defaults.items():
        setattr(u, k, v)
    return u


def test_uniform_layout_is_the_renderers(shading):
    import ctypes

    U = shading.BubbleUniform
    assert ctypes.sizeof(U) == 128
    assert U.edge_smoothing_mode.offset == 64 and U.patch_enabled.offset == 96 and U.padding.offset == 112


def test_drainage_profile_without_noise(orc, shading):
    # swirl_intensity = 0 turns off FBM, swirl noise and ripple: h = base (1 - 0.2 (1 - ny)(1 + p))
    for t in (0.0, 3.0, 50.0):
        u = _uniform(shading, swirl_intensity=0.0, film_time=t, base_thickness_nm=700.0)
        p = min(f32(t) * f32(0.5) * f32(0.1), 1.0)
        for ny in (-1.0, -0.3, 0.0, 0.6, 1.0):
            n = (math.sqrt(1 - ny * ny), ny, 0.0)
            want = 700.0 * (1 - 0.4 * (1 - ny) * 0.5 * (1 + p))
            assert abs(orc.film_thickness(u, n) - want) <= 1e-4 * 700, (t, ny)


def _top_fragment(orc, shading, lut, **kw):
    """One fragment at the top of the sphere seen from straight above (cos theta = 1)."""
    u = _uniform(shading, swirl_intensity=0.0, **kw)
    return orc.shade_fragments(u, (0.0, 1.0, 0.0), lut, [(0.0, 1.0, 0.0)], [(0.0, 0.025, 0.0)])[0]


def test_lut_texel_centres_and_black_film(orc, shading):
    lut = np.random.default_rng(2).integers(0, 256, (64, 256, 4), dtype=np.uint8)
    for k in (4, 5, 77, 200, 255):  # thickness >= 30 nm (k = 4: 35 nm)
        base = (k + 0.5) / 256 * 2000.0  # thickness at a texel centre; cos = 1 clamps to row 63
        rgba = _top_fragment(orc, shading, lut, base_thickness_nm=base, interference_intensity=1.0)
        want = np.minimum(lut[63, k, :3] / 255.0, 1.0) + np.array([0.95, 0.97, 1.0]) * 0.1
        np.testing.assert_allclose(rgba[:3], want, atol=2e-6)
        assert abs(rgba[3] - 0.3) < 1e-7  # edge 0: base alpha
    black = _top_fragment(orc, shading, lut, base_thickness_nm=25.0)
    np.testing.assert_allclose(black, [0.02, 0.02, 0.02, 0.15], atol=1e-7)


@pytest.mark.parametrize("mode", [0, 1, 2])
def test_edge_smoothing_alpha(orc, shading, mode):
    lut = np.zeros((64, 256, 4), np.uint8)
    u = _uniform(shading, swirl_intensity=0.0, edge_smoothing_mode=mode)
    for c in (0.0, 0.25, 0.5, 0.9):
        # a fragment on the equator seen along a direction at angle acos(c) to its normal
        n = (1.0, 0.0, 0.0)
        wp = (0.025, 0.0, 0.0)
        view = (c, 0.0, math.sqrt(1 - c * c))
        cam = (wp[0] + view[0], wp[1], wp[2] + view[2])
        a = orc.shade_fragments(u, cam, lut, [n], [wp])[0][3]
        e = 1 - c
        se = e if mode == 0 else (e * e * (3 - 2 * e) if mode == 1 else e ** 1.5)
        assert abs(a - (0.3 + 0.6 * se)) < 2e-6, (mode, c, a)


def test_frame_background_and_centre(orc, shading):
    lut = np.full((64, 256, 4), 128, np.uint8)
    u = _uniform(shading)
    cam = shading.Camera(aspect=1.0)
    rgba8, lin = orc.shade_frame(u, cam.view_proj(), cam.position(), 0.025, lut, 48, 48)
    # corners miss the bubble: the clear colour, sRGB-encoded, alpha 1
    bg = [0.1, 0.1, 0.15]
    np.testing.assert_allclose(lin[0, 0], bg + [1.0], atol=1e-7)
    enc = [round(255 * (1.055 * x ** (1 / 2.4) - 0.055)) for x in bg]
    assert list(rgba8[0, 0]) == enc + [255]
    # the centre pixel sees the bubble: a blend of the fragment over the background
    assert not np.allclose(lin[24, 24, :3], bg)
    assert abs(lin[24, 24, 3] - 1.0) < 1e-6
    # the bubble's silhouette: disc of radius ~ atan(0.025 / 0.2) / tan(fov / 2) of the half width
    hit = np.any(np.abs(lin[..., :3] - np.array(bg)) > 1e-6, axis=-1)
    frac = hit.mean()
    r = math.tan(math.asin(0.025 / 0.2)) / math.tan(math.radians(22.5))
    assert abs(frac - math.pi * r * r / 4) < 0.02


# --- the reference's camera.rs (:122-345) and BubbleUniform (pipeline.rs:2884-2955,
# headless.rs:566-571) tests, on the host-side mirrors ---------------------------------------------
def test_reference_camera(shading):
    C = shading.Camera
    cam = C(aspect=16 / 9)
    assert cam.distance > 0 and cam.fov > 0  # test_camera_creation
    cam = C(aspect=1.0)
    assert abs(np.linalg.norm(cam.position()) - cam.distance) < 1e-3  # test_camera_position
    for dx, sign in ((100.0, 1), (-100.0, -1)):  # test_orbit_increases_yaw / decreases
        c = C(aspect=1.0)
        y0 = c.yaw
        c.orbit(dx, 0.0)
        assert (c.yaw - y0) * sign > 0
    c = C(aspect=1.0)
    p0 = c.position()
    c.orbit(50.0, 50.0)
    assert np.linalg.norm(p0 - c.position()) > 1e-3  # test_orbit_changes_position
    for dy in (10000.0, -10000.0):  # test_pitch_clamping_upper / lower
        c = C(aspect=1.0)
        c.orbit(0.0, dy)
        assert abs(c.pitch) <= math.pi / 2 - 0.01 + 1e-12
    for d, smaller in ((2.0, True), (-2.0, False)):  # test_zoom_in / out
        c = C(aspect=1.0)
        d0 = c.distance
        c.zoom(d)
        assert (c.distance < d0) == smaller
    c = C(aspect=1.0)
    c.zoom(1000.0)
    assert c.distance >= 0.05  # test_zoom_min_bound
    c.zoom(-1000.0)
    assert c.distance <= 10.0  # test_zoom_max_bound
    c = C(aspect=16 / 9)
    c.set_aspect(4 / 3)
    assert abs(c.aspect - 4 / 3) < 1e-3  # test_aspect_ratio_update
    c = C(aspect=1.0)
    assert abs(np.linalg.det(c.view_matrix())) > 1e-3  # test_view_matrix_is_valid
    assert abs(np.linalg.det(c.projection_matrix())) > 1e-3  # test_projection_matrix_is_valid
    c = C(aspect=1.0)  # test_input_sequence_simulation
    p0 = c.position()
    for _ in range(10):
        c.orbit(10.0, 5.0)
    c.zoom(2.0)
    assert np.linalg.norm(p0 - c.position()) > 0.01
    assert abs(np.linalg.norm(c.position() - np.asarray(c.target)) - c.distance) < 1e-3
    c = C(aspect=1.0)  # test_orbit_360_degrees
    p0 = c.position()
    for _ in range(628):
        c.orbit(1.0, 0.0)
    assert np.linalg.norm(p0 - c.position()) < 0.1
    c = C(aspect=1.0)  # test_camera_uniform_contents
    vp, pos = c.uniform()
    np.testing.assert_allclose(pos, c.position(), atol=1e-3)
    np.testing.assert_allclose(vp.reshape(4, 4), c.view_projection_matrix().T, atol=1e-3)  # columns


def test_reference_bubble_uniform(shading):
    import ctypes

    U = shading.BubbleUniform
    u = U.default()  # test_bubble_uniform_default_values, headless.rs test_bubble_uniform_defaults
    for name, want in (("refractive_index", 1.33), ("base_thickness_nm", 500.0), ("interference_intensity", 4.0),
                       ("base_alpha", 0.3), ("edge_alpha", 0.6), ("film_time", 0.0), ("swirl_intensity", 1.0),
                       ("drainage_speed", 0.5), ("pattern_scale", 1.0)):
        assert abs(getattr(u, name) - want) < 1e-6, name
    for name, v in (("film_time", 10.0), ("swirl_intensity", 2.0), ("drainage_speed", 0.5), ("pattern_scale", 3.0)):
        setattr(u, name, v)  # test_bubble_uniform_film_dynamics_present
        assert abs(getattr(u, name) - v) < 1e-6
    assert ctypes.sizeof(U) == 128  # test_bubble_uniform_size_alignment
    for name, off in (("refractive_index", 0), ("base_thickness_nm", 4), ("time", 8), ("interference_intensity", 12),
                      ("base_alpha", 16), ("edge_alpha", 20), ("film_time", 36), ("swirl_intensity", 40),
                      ("drainage_speed", 44), ("pattern_scale", 48)):  # test_bubble_uniform_field_offsets
        assert getattr(U, name).offset == off, name
