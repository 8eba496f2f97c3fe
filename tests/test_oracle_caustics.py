"""The caustic-pass oracle (caustics_compute.wgsl restated in oracle/caustics.cpp) against closed
forms: a uniform film, a parabolic trough, a saddle (the Hessian branch factor), the periodic
phi wrap and the clamped theta border."""
import numpy as np
import pytest


@pytest.fixture(scope="module")
def cp():
    from soap_bubble_simulation_gb300 import caustics

    return caustics


def params(cp, w, h, **kw):
    p = cp.CausticParams()
    for k, v in dict(grid_width=w, grid_height=h, refractive_index=1.33, film_thickness_scale=1e6, light_dir_y=-1.0,
                     light_intensity=1.0, focal_length=0.1, caustic_intensity=2.0, caustic_sharpness=1.5,
                     branch_threshold=0.001, ground_y=-0.1, bubble_radius=0.025).items():
        setattr(p, k, v)
    for k, v in kw.items():
        setattr(p, k, v)
    return p


def test_uniform_film(orc, cp):
    p = params(cp, 40, 20)
    out = orc.caustics(p, np.full((20, 40), 5e-7, np.float32))
    np.testing.assert_allclose(out, 2.0, rtol=1e-6)


def test_parabolic_trough(orc, cp):
    w, h, a = 64, 16, 0.25  # a (x - 31)^2 exact in float32
    x = np.arange(w, dtype=np.float64)
    field = np.tile(a * (x - 31.0) ** 2, (h, 1)).astype(np.float32)
    p = params(cp, w, h, focal_length=0.5, caustic_sharpness=1.0, caustic_intensity=1.0)
    out = orc.caustics(p, field)
    for xi in range(2, w - 2):
        gx = 2 * a * (xi - 31.0)
        focusing = 1.0 / max(abs(1.0 + 2 * a * 0.5), 0.01)
        want = min(focusing * (1 + abs(gx) * 0.5), 10.0)
        assert abs(out[8, xi] - want) <= 1e-5 * want, (xi, out[8, xi], want)


def test_saddle_branches(orc, cp):
    w, h, a = 32, 32, 0.05
    yy, xx = np.mgrid[0:h, 0:w].astype(np.float64)
    field = (a * ((xx - 16) ** 2 - (yy - 16) ** 2)).astype(np.float32)
    p = params(cp, w, h, focal_length=0.0, caustic_sharpness=1.0, caustic_intensity=1.0)
    out = orc.caustics(p, field)
    # Hessian det = (2a)(-2a) = -0.01 < -0.001: branch factor 1.5, focusing 1, refraction at the
    # saddle point 1
    assert abs(out[16, 16] - 1.5) < 1e-6
    p.branch_threshold = 0.02  # det no longer below -threshold
    assert abs(orc.caustics(p, field)[16, 16] - 1.0) < 1e-6


def test_phi_wraps_and_theta_clamps(orc, cp):
    w, h = 16, 8
    field = np.zeros((h, w), np.float32)
    field[:, w - 1] = 1.0  # the left neighbour of column 0 through the periodic wrap
    p = params(cp, w, h, focal_length=0.0, caustic_sharpness=1.0, caustic_intensity=1.0, branch_threshold=10.0)
    out = orc.caustics(p, field)
    assert abs(out[4, 0] - (1 + 0.5 * 0.5)) < 1e-6  # |gx| = 1/2 at column 0
    field = np.zeros((h, w), np.float32)
    field[0, :] = 1.0  # row 0: its own upper neighbour (clamped)
    out = orc.caustics(p, field)
    assert abs(out[0, 5] - (1 + 0.5 * 0.5)) < 1e-6  # gy = (row1 - row0) / 2 = -1/2
    assert abs(out[1, 5] - (1 + 0.5 * 0.5)) < 1e-6  # gy = (row2 - row0) / 2 = -1/2
