"""Drainage surrogate on the GPU against the CPU oracle (include/sbs_nn.h restated in oracle/).

Bars: features bit-identical (the same FP32 operations); the network output within 1e-2 of
max |y| at every cell and 5e-4 in RMS (FP32 tensor-core accumulation order vs double: an
activation that lands within an FP32 rounding of a BF16 rounding boundary flips by one BF16 ulp,
2^-8 of itself - about 6e-5 of all activations, hundreds per 256 x 512 field - and the flip
propagates through the later layers, so the worst cell grows with the grid while the RMS stays
near 5e-5; the RMS bar catches any systematic error); gradients within 3e-2 relative L-inf per
layer (the per-layer BF16 gradients amplify those flips). Every network test runs with both
activations (GELU, hard-swish).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

LAYERS = [("W1", 0, 4608), ("b1", 4608, 4640), ("W2", 4640, 13856), ("b2", 13856, 13888), ("W3", 13888, 23104),
          ("b3", 23104, 23136), ("W4", 23136, 23424), ("b4", 23424, 23425)]


def fields(nf, nt, np_, seed):
    from soap_bubble_simulation_gb300 import synthetic as S

    hs, cs = [], []
    for k in range(nf):
        hs.append(S.smooth_modes(nt, np_, seed=seed + k))
        cs.append(S.surfactant_noise(nt, np_, seed=seed + 100 + k))
    return np.stack(hs).astype(np.float32), np.stack(cs).astype(np.float32)


def params_list(sbs, nf, nt, np_, seed):
    g = np.random.default_rng(seed)
    return [sbs.field_params(nt, np_, viscosity=float(10 ** g.uniform(-4, -2)),
                             bubble_radius=float(10 ** g.uniform(np.log10(0.0075), np.log10(0.04))))
            for _ in range(nf)]


def orc_params(orc, p):
    return orc.wgsl_params(dt=p.dt, gravity=p.gravity, viscosity=p.viscosity, density=p.density,
                           diffusion_coeff=p.diffusion_coeff, bubble_radius=p.bubble_radius,
                           grid_width=p.grid_width, grid_height=p.grid_height)


def check_y(y, want):
    scale = np.abs(want).max()
    err = np.abs(y - want).max() / scale
    rms = np.sqrt(np.mean((y.astype(np.float64) - want) ** 2)) / scale
    assert err <= 1e-2 and rms <= 5e-4, (err, rms)


@pytest.fixture(scope="module", params=["gelu", "hswish"])
def net(sbs, request):
    s = sbs.DrainageSurrogate(seed=11, activation=request.param)
    yield s
    s.close()


def test_activation_setting(sbs):
    s = sbs.DrainageSurrogate(seed=1)
    assert s.activation == "gelu"
    s.activation = "hswish"
    assert s.activation == "hswish"
    with pytest.raises(ValueError):
        s.activation = "relu"
    with pytest.raises(sbs.SbsError):
        sbs._native.call("sbs_surrogate_set_activation", s._h, 7)
    assert s.activation == "hswish"
    s.close()


@pytest.mark.parametrize("nt,np_", [(32, 64), (20, 200), (64, 128)])
def test_features_bit_identical(sbs, orc, net, nt, np_):
    h, c = fields(2, nt, np_, seed=5)
    ps = params_list(sbs, 2, nt, np_, seed=1)
    h[0, 3, 7] = np.nan  # non-finite input: clamped on both sides
    x = net.features(h, c, ps)
    for b in range(2):
        want = orc.nn_features(h[b], c[b], orc_params(orc, ps[b]))
        np.testing.assert_array_equal(x[b], want)


@pytest.mark.parametrize("nt,np_,nf", [(16, 32, 2), (24, 160, 1), (64, 256, 3)])
def test_forward_matches_oracle(sbs, orc, net, nt, np_, nf):
    h, c = fields(nf, nt, np_, seed=nt)
    ps = params_list(sbs, nf, nt, np_, seed=nt + 1)
    theta = net.params
    y = net.forward(h, c, ps, mode="layered")
    x = np.stack([orc.nn_features(h[b], c[b], orc_params(orc, ps[b])) for b in range(nf)])
    want = orc.nn_forward(theta, x, net.activation)
    check_y(y, want)


# 40 columns: one ragged chunk of the weight gradient per row with both phi seams; 136: three
# chunks, the last ragged; 128: two full chunks, the seam after a full one; 4 x 3: the smallest
# grid (both poles reflect into the same interior rows, three cells between the seams)
@pytest.mark.parametrize("nt,np_,nf", [(16, 40, 2), (12, 136, 2), (10, 128, 1), (4, 3, 2)])
def test_gradients_match_oracle(sbs, orc, net, nt, np_, nf):
    h, c = fields(nf, nt, np_, seed=3)
    ps = params_list(sbs, nf, nt, np_, seed=4)
    target = np.random.default_rng(9).standard_normal((nf, nt, np_)).astype(np.float32)
    loss, grad = net.loss_grad(h, c, ps, target)
    x = np.stack([orc.nn_features(h[b], c[b], orc_params(orc, ps[b])) for b in range(nf)])
    loss_o, grad_o = orc.nn_loss_grad(net.params, x, target, net.activation)
    assert abs(loss - loss_o) <= 1e-3 * loss_o
    for name, a, b in LAYERS:
        e = np.abs(grad[a:b] - grad_o[a:b]).max() / np.abs(grad_o[a:b]).max()
        assert e <= 3e-2, (name, e)


def trained_surrogate(sbs, ntraj=24, nt=48, np_=96, iters=300, activation="gelu"):
    s = sbs.DrainageSurrogate(seed=3, activation=activation)
    g = np.random.default_rng(0)
    from soap_bubble_simulation_gb300 import synthetic as S

    for k in range(ntraj):
        p = sbs.field_params(nt, np_, viscosity=float(10 ** g.uniform(-4, -2)),
                             bubble_radius=float(10 ** g.uniform(np.log10(0.0075), np.log10(0.04))))
        s.add_trajectory(S.smooth_modes(nt, np_, seed=1000 + k), S.surfactant_noise(nt, np_, seed=2000 + k), p,
                         pairs=3)
    losses = s.train(ntraj - 4, iters, batch=4, lr=3e-3, seed=1)
    return s, losses


@pytest.mark.parametrize("activation", ["gelu", "hswish"])
def test_training_beats_identity(sbs, activation):
    s, losses = trained_surrogate(sbs, activation=activation)
    assert np.isfinite(losses).all()
    assert losses[-20:].mean() < 0.2 * losses[:5].mean()
    ev = s.evaluate(20, 4, mode="layered")
    # the trained network predicts the 64-pass change: far below the error of doing nothing
    assert ev["loss"] < 0.1 * ev["loss_identity"], ev
    assert ev["rel_linf"] < 0.5 * ev["rel_linf_identity"], ev
    s.close()


def test_rollout_checks_and_fallback(sbs):
    s, _ = trained_surrogate(sbs, ntraj=8, iters=100)
    from soap_bubble_simulation_gb300 import synthetic as S

    nt, np_ = 48, 96
    p = sbs.field_params(nt, np_, bubble_radius=0.02)
    sim = sbs.GPUDrainageSimulator(None, 500e-9, np_, nt)
    sim.update_params(p)
    h0, c0 = S.smooth_modes(nt, np_, seed=77), S.surfactant_noise(nt, np_, seed=78)
    sim.set_thickness_array(h0)
    sim.set_concentration_array(c0)
    st = s.rollout(sim, 8 * 64, check_every=2, tol=1e-3, mode="layered")
    assert st["rollouts"] == 8 and st["checks"] == 4 and st["plain"] == 4 and st["surrogate"] == 4
    assert st["failed_checks"] == 0 and st["max_check_error"] < 1e-3
    h_sur = sim.thickness_array()
    ref = sbs.GPUDrainageSimulator(None, 500e-9, np_, nt)
    ref.update_params(p)
    ref.set_thickness_array(h0)
    ref.set_concentration_array(c0)
    ref.run(8 * 64)
    assert sbs.masked_error(h_sur, ref.thickness_array()) < 1e-3
    # an impossible tolerance: every check fails and the plain solver runs the fallback intervals
    st = s.rollout(sim, 8 * 64, check_every=4, tol=1e-30, mode="layered")
    assert st["checks"] == 2 and st["failed_checks"] == 2 and st["plain"] == 8 and st["surrogate"] == 0
    s.close()


@pytest.mark.parametrize("nt,np_,nf", [(16, 32, 2), (20, 200, 1), (21, 96, 1), (64, 256, 3), (256, 512, 1), (37, 130, 2)])
def test_fused_forward_matches_oracle(sbs, orc, net, nt, np_, nf):
    """The fused tcgen05 kernel: narrow grids whose strip wraps, partial strips, several row blocks."""
    h, c = fields(nf, nt, np_, seed=nt + 7)
    ps = params_list(sbs, nf, nt, np_, seed=nt + 8)
    y = net.forward(h, c, ps, mode="fused")
    x = np.stack([orc.nn_features(h[b], c[b], orc_params(orc, ps[b])) for b in range(nf)])
    want = orc.nn_forward(net.params, x, net.activation)
    check_y(y, want)
    check_y(y, net.forward(h, c, ps, mode="layered"))


def test_fused_advance_matches_layered(sbs, net):
    from soap_bubble_simulation_gb300 import synthetic as S

    nt, np_ = 96, 192
    p = sbs.field_params(nt, np_, bubble_radius=0.02)
    out = {}
    for mode in ("layered", "fused"):
        sim = sbs.GPUDrainageSimulator(None, 500e-9, np_, nt)
        sim.update_params(p)
        sim.set_thickness_array(S.smooth_modes(nt, np_, seed=5))
        sim.set_concentration_array(S.surfactant_noise(nt, np_, seed=6))
        net.advance(sim, mode=mode)
        out[mode] = sim.thickness_array()
    d = np.abs(out["fused"] - out["layered"]).max()
    assert d <= 1e-12, d  # kout * |dy| ~ 1e-13 m per unit of y
