"""Pins the interference oracle: the reference's interference.rs (612-792) and
interference_lut.rs (165-205) unit tests, plus closed-form checks. CPU only."""
import math

import numpy as np
import pytest

EPS = 1e-6


def test_rgb_color_clamping():
    from soap_bubble_simulation_gb300 import RgbColor

    c = RgbColor.new(1.5, -0.5, 0.5)
    assert abs(c.red - 1.0) < EPS and abs(c.green) < EPS and abs(c.blue - 0.5) < EPS


def test_rgb_color_to_u8():
    from soap_bubble_simulation_gb300 import RgbColor

    assert RgbColor.new(1.0, 0.5, 0.0).to_u8_tuple() == (255, 128, 0)


def test_transmission_angle_normal_incidence(orc):
    assert abs(orc.transmission_angle_cos(1.33, 1.0) - 1.0) < EPS


def test_transmission_angle_snells_law(orc):
    ci = math.sqrt(2.0) / 2.0
    ct = orc.transmission_angle_cos(1.5, ci)
    si, st = math.sqrt(1 - ci * ci), math.sqrt(1 - ct * ct)
    assert abs(si / st - 1.5) < 1e-4


def test_fresnel_normal_incidence(orc):
    expected = ((1.0 - 1.33) / (1.0 + 1.33)) ** 2
    assert abs(orc.fresnel(1.33, 1.0)[2] - expected) < 1e-4


def test_zero_thickness_gives_zero_intensity(orc):
    assert abs(orc.reflected_intensity(1.33, 0.0, 1.0, 550.0)) < EPS


@pytest.mark.parametrize("t", [100.0, 200.0, 300.0, 400.0, 500.0])
def test_interference_produces_colors(orc, t):
    assert orc.interference_color(1.33, t, 1.0).max() > 0.01


def test_color_varies_with_thickness(orc):
    assert np.abs(orc.interference_color(1.33, 100, 1.0) - orc.interference_color(1.33, 300, 1.0)).sum() > 0.01


def test_color_varies_with_angle(orc):
    assert np.abs(orc.interference_color(1.33, 300, 1.0) - orc.interference_color(1.33, 300, 0.5)).sum() > 0.001


def test_lookup_table_generation(orc):
    t = orc.lut1d(1.33, 0.0, 1000.0, 100, 1.0)
    assert t.shape == (100, 3)
    assert np.all((t >= 0) & (t <= 1))


def test_2d_lookup_table_generation(orc):
    t = orc.lut2d(1.33, 0.0, 500.0, 10, 5)
    assert t.shape == (10, 5, 3)


def test_linear_vs_gamma_color(orc):
    lin = orc.interference_color(1.33, 300.0, 1.0, gamma=False)
    gam = orc.interference_color(1.33, 300.0, 1.0, gamma=True)
    if 0.01 < lin[0] < 0.99:
        assert gam[0] >= lin[0]


def test_custom_wavelengths(orc):
    c = orc.interference_color(1.33, 300.0, 1.0, wl=(700.0, 550.0, 400.0))
    assert np.all((c >= 0) & (c <= 1))


def test_intensity_closed_form(orc):
    """Normal incidence: I = 2R(1-cos d)/(1+R^2-2R cos d), d = 2 pi (2 n t + l/2)/l."""
    n, t, wl = 1.33, 250.0, 600.0
    R = ((1 - n) / (1 + n)) ** 2
    d = 2 * math.pi * (2 * n * t + wl / 2) / wl
    want = 2 * R * (1 - math.cos(d)) / (1 + R * R - 2 * R * math.cos(d))
    assert orc.reflected_intensity(n, t, 1.0, wl) == pytest.approx(want, rel=1e-12)


def test_lut2d_matches_scalar(orc):
    lut = orc.lut2d(1.33, 0.0, 1000.0, 256, 64)
    i, j = 77, 41
    want = orc.interference_color(1.33, 0.0 + i * ((1000.0 - 0.0) / 255), j * (1.0 / 63))
    np.testing.assert_array_equal(lut[i, j], want)


# --- interference_lut.rs:170-204 ------------------------------------------------------------------
def test_lut_generation_produces_valid_data(orc):
    lut = orc.interference_lut_rgba8(1.33, 1.0)
    assert lut.size == 256 * 64 * 4
    assert np.all(lut.reshape(-1, 4)[:, 3] == 255)


def test_thin_film_produces_colors(orc):
    rgb = orc.thin_film_interference7(500.0, 0.9, 1.33, 1.0)
    assert np.all((rgb >= 0) & (rgb <= 1))
    assert rgb.sum() > 0.01


def test_lut_snells_law(orc):
    assert abs(orc.lut_snells_law(1.0, 1.33) - 1.0) < 0.01
    ct = orc.lut_snells_law(0.1, 1.33)
    assert 0.0 < ct < 1.0


def test_lut_fresnel_at_normal_incidence(orc):
    r = orc.lut_fresnel_unpolarized(1.0, 1.0, 1.0, 1.33)
    assert 0.01 < r < 0.05


def test_lut_layout_angle_major(orc):
    """Row a (cos = a/63) of the RGBA8 table equals thin_film_interference at that angle."""
    lut = orc.interference_lut_rgba8(1.33, 1.0).reshape(64, 256, 4)
    a, t = 50, 100
    rgb = orc.thin_film_interference7(np.float32(t) / np.float32(255) * np.float32(2000), np.float32(a) / np.float32(63),
                                      1.33, 1.0)
    want = (np.clip(rgb, 0, 1) * np.float32(255)).astype(np.uint8)
    np.testing.assert_array_equal(lut[a, t, :3], want)


# --- wall.wgsl:176-207 -------------------------------------------------------------------------
def test_schlick_normal_incidence(orc):
    """At cos = 1 Schlick reduces to R0 and the transmitted Airy term to 1/(1 + F sin^2(d/2))."""
    n, t, wl = 1.33, 300.0, 532.0
    r0 = ((1 - n) / (1 + n)) ** 2
    F = 4 * r0 / (1 - r0) ** 2
    d = 2 * math.pi * 2 * n * t / wl + math.pi
    want = 1.0 / (1.0 + F * math.sin(d / 2) ** 2)
    assert orc.schlick_interference(t, wl, 1.0, n) == pytest.approx(want, rel=1e-5)


def test_lut_sample_hits_texel_centres(orc):
    """Sampling at a texel centre returns that texel (bubble.wgsl:425-439 with a linear sampler)."""
    lut = orc.interference_lut_rgba8(1.33, 1.0).reshape(64, 256, 4)
    i, j = 120, 30
    t = (i + 0.5) / 256 * 2000.0
    c = (j + 0.5) / 64
    got = orc.lut_rgba8_sample(lut, 256, 64, t, c)
    np.testing.assert_allclose(got, lut[j, i, :3] / 255.0, atol=1e-6)


def test_spectral_reduces_to_lut_formulation(orc):
    """orc_spectral_rgb with 7 wavelengths and the CIE weights /7 equals the LUT's XYZ sum."""
    wl = np.array([400.0, 450.0, 500.0, 550.0, 600.0, 650.0, 700.0])
    cmf = np.eye(3)[np.zeros(7, dtype=int)] * 0 + 1.0 / 7  # flat weights
    out = orc.spectral_rgb(np.array([500.0], np.float32), np.array([0.9], np.float32), np.array([1.33], np.float32),
                           wl, cmf)
    assert np.all(out >= 0) and out[0, 0] == pytest.approx(out[0, 1])
