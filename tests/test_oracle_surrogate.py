"""The surrogate oracle (include/sbs_nn.h restated on the CPU) pinned by analytic checks: the
GELU polynomial against x * normal CDF, hard-swish against its closed form, the finite-difference
features against closed-form derivatives, and the backward pass against central finite
differences of the forward pass (exact mode), for both activations."""
import math

import numpy as np
import pytest
from scipy.special import erf

S2 = 1e-5


def test_gelu_polynomial_and_derivative(orc):
    xs = np.linspace(-6, 6, 241)
    g = np.array([orc.nn_gelu(v) for v in xs])
    gt = xs * 0.5 * (1 + erf(xs / math.sqrt(2)))
    assert np.abs(g - gt).max() < 4.1e-3
    assert abs(orc.nn_gelu(-3.5)) < 1e-6 and abs(orc.nn_gelu(3.5) - 3.5) < 1e-6
    pts = np.concatenate([np.linspace(-5, -3.05, 9), np.linspace(-2.95, 2.95, 31), np.linspace(3.05, 5, 9)])
    fd = np.array([(orc.nn_gelu(v + 1e-2) - orc.nn_gelu(v - 1e-2)) / 2e-2 for v in pts])
    gd = np.array([orc.nn_gelu_grad(v) for v in pts])
    assert np.abs(fd - gd).max() < 2e-4


def test_hardswish_and_derivative(orc):
    xs = np.linspace(-6, 6, 241)
    a = np.array([orc.nn_hswish(v) for v in xs])
    want = xs * np.clip(xs / 6 + 0.5, 0, 1)
    assert np.abs(a - want).max() <= 1e-6 * np.abs(xs).max()
    assert orc.nn_hswish(-3.5) == 0.0 and orc.nn_hswish(3.5) == 3.5
    assert math.isnan(orc.nn_hswish(float("nan")))
    # away from the kinks at +-3 the derivative matches central differences
    pts = np.concatenate([np.linspace(-5, -3.05, 9), np.linspace(-2.95, 2.95, 31), np.linspace(3.05, 5, 9)])
    fd = np.array([(orc.nn_hswish(v + 1e-2) - orc.nn_hswish(v - 1e-2)) / 2e-2 for v in pts])
    gd = np.array([orc.nn_hswish_grad(v) for v in pts])
    assert np.abs(fd - gd).max() < 2e-4
    assert orc.nn_hswish_grad(-4.0) == 0.0 and orc.nn_hswish_grad(4.0) == 1.0 and orc.nn_hswish_grad(0.0) == 0.5


def _params(orc, nt, np_, **kw):
    return orc.wgsl_params(grid_width=np_, grid_height=nt, **kw)


def test_features_match_closed_form_derivatives(orc):
    nt, np_ = 129, 256
    th = np.linspace(0, np.pi, nt)[:, None]
    ph = (2 * np.pi / np_) * np.arange(np_)[None, :]
    A = 40e-9
    p = _params(orc, nt, np_, bubble_radius=0.025, viscosity=2e-3)
    c = np.full((nt, np_), 0.55, np.float32)
    rows = slice(20, nt - 20)
    # theta curvature and cot(theta)-weighted slope of h = H0 + A sin(2 theta)
    h = (550e-9 + A * np.sin(2 * th) + 0 * ph).astype(np.float32)
    x = orc.nn_features(h, c, p)
    want1 = -4 * A * np.sin(2 * th) / S2
    with np.errstate(divide="ignore"):
        want3 = np.cos(th) / np.sin(th) * 2 * A * np.cos(2 * th) / S2
    assert np.abs(x[rows, :, 1] - want1[rows]).max() < 5e-3 * np.abs(want1).max()  # BF16: 2^-9 relative
    assert np.abs(x[rows, :, 3] - want3[rows]).max() < 5e-3 * np.abs(want3[rows]).max()
    # phi curvature / sin^2 of h = H0 + A cos(3 phi)
    h = (550e-9 + A * np.cos(3 * ph) + 0 * th).astype(np.float32)
    x = orc.nn_features(h, c, p)
    with np.errstate(divide="ignore"):
        want2 = -9 * A * np.cos(3 * ph) / np.sin(th) ** 2 / S2
    assert np.abs(x[rows, :, 2] - want2[rows]).max() < 6e-3 * np.abs(want2[rows]).max()
    # level, surfactant, log-viscosity, log-diameter, gravity feature
    R, eta = 0.025, 2e-3
    hc = x[:, :, 0] * 150e-9 + 550e-9
    assert np.abs(hc - h).max() < 2e-9
    assert np.allclose(x[:, :, 4], 0.5, atol=4e-3)
    assert np.allclose(x[:, :, 5], np.log10(eta / 1e-3), rtol=1e-2)
    assert np.allclose(x[:, :, 6], 3 * np.log10(2 * R / 0.035), rtol=1e-2)
    gk = -(1000 * 9.81 / (3 * eta)) / (1e-9 / R**2 * S2)
    want7 = gk * np.sin(th) * h.astype(np.float64) ** 3
    assert np.abs(x[:, :, 7] - want7).max() < 1e-2 * np.abs(want7).max()
    kout = orc.nn_kout(p)
    mu = 64 * 1e-3 * 1e-9 / R**2
    assert abs(kout - mu * S2) < 1e-6 * kout
    # diffusion numbers of the 64-pass interval and the latitude
    dth, dph = np.pi / (nt - 1), 2 * np.pi / np_
    assert np.allclose(x[:, :, 8], np.log10(mu / dth**2 / 0.044), atol=2e-2)
    se = np.maximum(np.sin(th), 0.05)
    assert np.allclose(x[:, :, 9], np.log10(mu / (dph**2 * se**2) / 0.044) + 0 * ph, atol=2e-2)
    assert np.allclose(x[:, :, 10], np.sin(th) + 0 * ph, atol=4e-3)
    assert (x[:, :, 11:] == 0).all()


def test_features_are_finite_for_nonfinite_input(orc):
    nt, np_ = 16, 32
    h = np.full((nt, np_), 500e-9, np.float32)
    h[1, 3] = np.nan
    h[2, 5] = np.inf
    x = orc.nn_features(h, np.full_like(h, 0.5), _params(orc, nt, np_))
    assert np.isfinite(x).all() and np.abs(x).max() <= 1e4


@pytest.mark.parametrize("act", ["gelu", "hswish"])
@pytest.mark.parametrize("nb,nt,np_", [(2, 6, 8), (1, 9, 12)])
def test_backward_matches_finite_differences(orc, nb, nt, np_, act):
    g = np.random.default_rng(nb * 100 + nt)
    theta = (0.08 * g.standard_normal(orc.NN_PARAMS)).astype(np.float32)
    x = g.standard_normal((nb, nt, np_, 16)).astype(np.float32)
    target = g.standard_normal((nb, nt, np_)).astype(np.float32)
    orc.nn_set_exact(True)
    try:
        loss, grad = orc.nn_loss_grad(theta, x, target, act)
        # parameters in every layer: weights at the reflected (dy = -1 / +1) and periodic taps, biases
        idx = np.concatenate([g.integers(0, 4608, 6), [4608, 4639], g.integers(4640, 13856, 6), [13856],
                              g.integers(13888, 23104, 6), [23104], g.integers(23136, 23424, 6), [23424]])
        for k in idx:
            eps = 1e-5
            tp, tm = theta.copy(), theta.copy()
            tp[k] += eps
            tm[k] -= eps
            fd = (orc.nn_loss_grad(tp, x, target, act)[0] - orc.nn_loss_grad(tm, x, target, act)[0]) / (2 * eps)
            # the step itself is float32-rounded: use the exact difference of the stored values
            fd *= 2 * eps / (float(tp[k]) - float(tm[k]))
            assert abs(fd - grad[k]) <= 1e-4 * max(1.0, abs(fd)) + 1e-6, (k, fd, grad[k])
    finally:
        orc.nn_set_exact(False)
    assert loss > 0


def test_apply_freezes_poles_and_clamps(orc):
    nt, np_ = 8, 16
    h = np.full((nt, np_), 100e-9, np.float32)
    y = np.full((nt, np_), -5.0, np.float32)
    out = orc.nn_apply(h, y, 3e-8)
    assert (out[0] == h[0]).all() and (out[-1] == h[-1]).all()
    assert (out[1:-1] == 0).all()
    out = orc.nn_apply(h, -y, 1e-9)
    assert np.allclose(out[1:-1], 100e-9 + 5e-9, rtol=1e-6)
