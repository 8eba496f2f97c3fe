"""The caustic pass on the GPU (sbs_caustics, sbs_gpu_drainage_caustics) against the oracle.
Bar: 2e-6 relative (every operation but pow is the same FP32 sequence; pow agrees to its rounding)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def cp(sbs):
    from soap_bubble_simulation_gb300 import caustics

    return caustics


def close(a, b):
    return np.abs(a - b).max() <= 2e-6 * max(1.0, float(np.abs(b).max()))


@pytest.mark.parametrize("h,w", [(64, 128), (33, 97), (7, 5), (512, 1024)])
def test_map_matches_oracle(sbs, orc, cp, h, w):
    from soap_bubble_simulation_gb300 import synthetic as S

    field = (S.smooth_modes(h, w, seed=h) * 1e9).astype(np.float32) / 50.0  # nm / 50: curvatures of order 1
    for kw in ({}, {"focal_length": 0.5, "caustic_sharpness": 2.3}, {"branch_threshold": 0.0}):
        p = cp.CausticParams.default(w, h)
        for k, v in kw.items():
            setattr(p, k, v)
        assert close(cp.caustic_map(p, field), orc.caustics(p, field)), kw


def test_pitched_device_input(sbs, orc, cp):
    import ctypes

    import torch

    N = sbs._native
    h, w, pitch = 48, 100, 128
    g = np.random.default_rng(0)
    field = g.normal(size=(h, w)).astype(np.float32)
    padded = np.zeros((h, pitch), np.float32)
    padded[:, :w] = field
    din = torch.from_numpy(padded).cuda()
    dout = torch.empty((h, w), device="cuda")
    p = cp.CausticParams.default(w, h)
    N.call("sbs_caustics", ctypes.cast(ctypes.byref(p), ctypes.c_void_p), ctypes.c_void_p(din.data_ptr()), pitch,
           ctypes.c_void_p(dout.data_ptr()), N.MEM_DEVICE, None)
    torch.cuda.synchronize()
    assert close(dout.cpu().numpy(), orc.caustics(p, field))


def test_simulator_field_without_copy(sbs, orc, cp):
    from soap_bubble_simulation_gb300 import synthetic as S

    nt, np_ = 64, 128
    h0 = S.smooth_modes(nt, np_, seed=5).astype(np.float32)
    c0 = S.surfactant_noise(nt, np_, seed=6)

    def sim(passes):
        s = sbs.GPUDrainageSimulator(None, 500e-9, np_, nt)
        s.set_thickness_array(h0)
        s.set_concentration_array(c0)
        s.run(passes)
        return s

    a, b = sim(9), sim(8)
    p = cp.CausticParams.default(np_, nt)
    p.focal_length = 2e5  # thickness in metres: curvatures ~1e-11 per cell^2
    assert close(a.caustic_map(p), orc.caustics(p, a.thickness_array()))
    # which = 1: the buffer the reference binds, one pass behind the newest field
    assert close(a.caustic_map(p, which=1), orc.caustics(p, b.thickness_array()))
    with pytest.raises(sbs.SbsError):
        a.caustic_map(cp.CausticParams.default(np_ + 1, nt))
    a.close()
    b.close()


def _vivid(cp, w, h):
    """Parameters under which a drained film's 1e-9-scale curvatures give a map that varies (both
    branch factors, focusing well away from 1)."""
    p = cp.CausticParams.default(w, h)
    p.focal_length = 2e8
    p.branch_threshold = 1e-21
    p.caustic_sharpness = 2.3
    return p


@pytest.mark.parametrize("nt,np_,marangoni", [(10, 40, False), (37, 132, True), (130, 600, False), (256, 512, True),
                                              (2048, 4096, False)])
def test_run_caustic_map_fused_equals_separate_pass(sbs, orc, cp, nt, np_, marangoni):
    """run_caustic_map (the map written by the run's final blocked launch) against run() followed
    by the separate caustic pass over the buffer the renderer binds: the same map and the same
    fields bit for bit, for runs too short to fuse (3 passes), just long enough (4), with a
    single-pass remainder (7), several blocked launches (12, 300) and several chunks (600); the
    map also within the caustic bar of the oracle."""
    from soap_bubble_simulation_gb300 import synthetic as S

    h0 = S.smooth_modes(nt, np_, seed=nt).astype(np.float32)
    c0 = S.surfactant_noise(nt, np_, seed=nt + 1)
    p = _vivid(cp, np_, nt)

    def fresh():
        sim = sbs.GPUDrainageSimulator(None, 500e-9, np_, nt)
        params = sbs.field_params(nt, np_, bubble_radius=0.02)
        params.marangoni_enabled = 1 if marangoni else 0
        sim.update_params(params)
        sim.set_thickness_array(h0)
        sim.set_concentration_array(c0)
        return sim

    passes_list = (3, 4, 7, 12, 300, 600) if nt <= 256 else (4, 100)
    fused, sep = fresh(), fresh()
    for passes in passes_list:
        m_f = fused.run_caustic_map(passes, p)
        sep.run(passes)
        m_s = sep.caustic_map(p, which=1)
        np.testing.assert_array_equal(m_f, m_s)
        np.testing.assert_array_equal(fused.thickness_array(), sep.thickness_array())
        np.testing.assert_array_equal(fused.concentration_array(), sep.concentration_array())
    assert m_f.std() > 1e-3 * np.abs(m_f).max(), "the map should vary"
    behind = fresh()
    behind.run(sum(passes_list) - 1)  # the field the last map was made from
    assert close(m_f, orc.caustics(p, behind.thickness_array()))


def test_step_caustic_map_fused_equals_separate_pass(sbs, cp):
    """The frame form: step(frame_dt) (steps_per_frame passes, the frame clock) and the map, fused,
    equals step() then caustic_map(which=1); with the simulator disabled only the map is made."""
    from soap_bubble_simulation_gb300 import synthetic as S

    nt, np_ = 96, 192
    p = _vivid(cp, np_, nt)
    sims = []
    for _ in range(2):
        sim = sbs.GPUDrainageSimulator(None, 500e-9, np_, nt)
        sim.set_thickness_array(S.smooth_modes(nt, np_, seed=3).astype(np.float32))
        sim.enabled = True
        sims.append(sim)
    a, b = sims
    for _ in range(3):
        m_a = a.step_caustic_map(1.0 / 60.0, p)
        b.step(1.0 / 60.0)
        m_b = b.caustic_map(p, which=1)
        np.testing.assert_array_equal(m_a, m_b)
        np.testing.assert_array_equal(a.thickness_array(), b.thickness_array())
        assert a.current_time() == b.current_time()
    a.enabled = False
    b.enabled = False
    np.testing.assert_array_equal(a.step_caustic_map(1.0 / 60.0, p), b.caustic_map(p, which=1))
    assert a.current_time() == b.current_time()
