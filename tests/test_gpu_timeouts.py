"""The bounded device waits, made to run out on purpose: each call reports SBS_E_TIMEOUT, its
kernel exits cleanly (no CUDA error, the context stays usable) and the next call on the same
handle or function computes the right result.

Nothing is faulted or hung: a host switch (sbs_set_stall_injection) makes the waits
unsatisfiable - the tensor-core kernels issue neither their MMAs nor the commits that would
signal them, so no asynchronous operation is outstanding when a wait expires, and the foam
kernel's grid barrier and the pole-ring barrier of the blocked DrainageSimulator step expect one
arrival more than there are blocks - and a short wait limit
(sbs_set_wait_limit, 2e5 cycles, ~0.1 ms) bounds every wait.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture
def short_waits(sbs):
    N = sbs._native
    old = ctypes.c_uint64()
    N.call("sbs_wait_limit", ctypes.byref(old))
    N.call("sbs_set_wait_limit", 200_000)
    yield N
    N.call("sbs_set_stall_injection", 0)
    N.call("sbs_set_wait_limit", old.value)


def test_wait_limit_arguments(sbs):
    N = sbs._native
    with pytest.raises(sbs.SbsError, match="wait limit"):
        N.call("sbs_set_wait_limit", 10)
    with pytest.raises(sbs.SbsError, match="stall"):
        N.call("sbs_set_stall_injection", 8)
    out = ctypes.c_uint64()
    N.call("sbs_wait_limit", ctypes.byref(out))
    assert out.value == 2_000_000_000


def test_spectral_tensor_core_wait_times_out_then_recovers(sbs, orc, short_waits):
    from soap_bubble_simulation_gb300 import synthetic

    N = short_waits
    t, ci, nf = synthetic.spectral_points(20_000, seed=11)
    wl = synthetic.WAVELENGTHS_81
    cmf = synthetic.spectral_cmf(wl)
    N.call("sbs_set_stall_injection", N.STALL_TENSOR_COMMITS)
    with pytest.raises(sbs.SbsError) as e:
        sbs.spectral_rgb(t, ci, nf, wl, cmf, mode="tc")
    assert e.value.code == N.SBS_E_TIMEOUT
    N.call("sbs_set_stall_injection", 0)
    got = sbs.spectral_rgb(t, ci, nf, wl, cmf, mode="tc")
    want = orc.spectral_rgb(t, ci, nf, wl, cmf)
    assert np.abs(got - want).max() / np.abs(want).max() <= 1e-2


def test_foam_grid_barrier_times_out_then_recovers(sbs, short_waits):
    from soap_bubble_simulation_gb300 import synthetic as S

    N = short_waits
    res = [32, 64, 96, 48]
    rad = np.array([0.01, 0.02, 0.03, 0.015], np.float32)
    foam = sbs.FoamDrainage(res, rad)
    hs = S.foam_fields(np.asarray(res, dtype=np.uint32), seed=3)

    def load():
        for b, r in enumerate(res):
            foam.set_thickness(b, hs[b])
            foam.set_concentration(b, np.full((r, 2 * r), 0.5, np.float32))

    load()
    foam.set_tiles(4, 32)
    N.call("sbs_set_stall_injection", N.STALL_GRID_BARRIER)
    with pytest.raises(sbs.SbsError) as e:
        foam.run(12)  # three phases of 4 steps: a barrier after each of the first two
    assert e.value.code == N.SBS_E_TIMEOUT
    N.call("sbs_set_stall_injection", 0)
    load()
    foam.run(12)
    for b, r in enumerate(res):
        sim = sbs.GPUDrainageSimulator(None, 500e-9, 2 * r, r)
        sim.set_bubble_radius(float(rad[b]))
        sim.set_thickness_array(hs[b])
        sim.run(12)
        np.testing.assert_array_equal(foam.thickness(b), sim.thickness_array())
    foam.close()


def test_fused_surrogate_wait_times_out_then_recovers(sbs, orc, short_waits):
    from soap_bubble_simulation_gb300 import synthetic

    N = short_waits
    nt, np_ = 40, 80
    net = sbs.DrainageSurrogate(seed=5)
    h = synthetic.smooth_modes(nt, np_, seed=10).astype(np.float32)[None]
    c = synthetic.surfactant_noise(nt, np_, seed=20)[None]
    p = [sbs.field_params(nt, np_, bubble_radius=0.02)]
    N.call("sbs_set_stall_injection", N.STALL_TENSOR_COMMITS)
    with pytest.raises(sbs.SbsError) as e:
        net.forward(h, c, p, mode="fused")
    assert e.value.code == N.SBS_E_TIMEOUT
    N.call("sbs_set_stall_injection", 0)
    y = net.forward(h, c, p, mode="fused")
    x = orc.nn_features(h[0], c[0], orc.wgsl_params(grid_width=np_, grid_height=nt, bubble_radius=0.02))[None]
    want = orc.nn_forward(net.params, x)
    assert np.abs(y - want).max() / np.abs(want).max() <= 1e-2
    net.close()


def test_blocked_drainage_pole_ring_barrier_times_out_then_recovers(sbs, short_waits):
    """The polar strips of the blocked DrainageSimulator step meet at a barrier per step; with it
    unsatisfiable the call reports the timeout, and afterwards the handle steps like a fresh one."""
    from soap_bubble_simulation_gb300 import synthetic

    N = short_waits
    cfg = sbs.SimulationConfig()
    cfg.resolution = 64
    h0 = np.ascontiguousarray(synthetic.bubble_c0(64, seed=2))

    def load(sim):
        N.call("sbs_drainage_set_thickness_f64", sim.handle, N.dptr(h0), h0.size)

    def field(sim):
        out = np.empty(h0.size)
        N.call("sbs_drainage_get_thickness_field_f64", sim.handle, N.dptr(out), out.size)
        return out

    sim, fresh = sbs.DrainageSimulator(cfg), sbs.DrainageSimulator(cfg)
    kb = ctypes.c_int()
    N.call("sbs_drainage_time_blocking", sim.handle, ctypes.byref(kb))
    assert kb.value > 1
    load(sim)
    N.call("sbs_set_stall_injection", N.STALL_GRID_BARRIER)
    with pytest.raises(sbs.SbsError) as e:
        sim.step_n(0.001, 4 * kb.value)
    assert e.value.code == N.SBS_E_TIMEOUT
    N.call("sbs_set_stall_injection", 0)
    fresh.step_n(0.001, 4 * kb.value)  # the same clock (fronts depend on it)
    for s in (sim, fresh):
        load(s)
        s.step_n(0.001, 16)
    np.testing.assert_array_equal(field(sim), field(fresh))


def test_training_convolution_waits_time_out_then_recover(sbs, short_waits):
    """The tensor-core training convolutions: with their commits withheld the training step reports
    the timeout; afterwards the same handle trains and its loss falls."""
    from soap_bubble_simulation_gb300 import synthetic as S

    N = short_waits
    nt, np_ = 32, 64
    s = sbs.DrainageSurrogate(seed=3)
    g = np.random.default_rng(0)
    for k in range(4):
        p = sbs.field_params(nt, np_, viscosity=float(10 ** g.uniform(-4, -2)), bubble_radius=0.02)
        s.add_trajectory(S.smooth_modes(nt, np_, seed=10 + k), S.surfactant_noise(nt, np_, seed=20 + k), p, pairs=2)
    N.call("sbs_set_stall_injection", N.STALL_TENSOR_COMMITS)
    with pytest.raises(sbs.SbsError) as e:
        s.train(4, 3, batch=2, lr=3e-3, seed=1)
    assert e.value.code == N.SBS_E_TIMEOUT
    N.call("sbs_set_stall_injection", 0)
    losses = s.train(4, 60, batch=2, lr=3e-3, seed=1)
    assert np.isfinite(losses).all() and losses[-10:].mean() < losses[:3].mean()
    s.close()
