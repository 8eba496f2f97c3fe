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
