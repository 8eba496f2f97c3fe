"""Branched flow on the GPU (sbs_branched_flow) against the oracle's literal restatement of
branched_flow_compute.wgsl: the texture bit for bit. Every operation is the same FP32 sequence on
both sides (acos / atan2 / exp included: the library's own published approximations) and the
deposits are integer atomic adds, whose order does not matter."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def br(sbs):
    from soap_bubble_simulation_gb300 import branched

    return branched


def field(nt=64, np_=128, seed=3, scale=1.0):
    from soap_bubble_simulation_gb300 import synthetic as S

    return (S.smooth_modes(nt, np_, seed=seed) * scale).astype(np.float32)


@pytest.mark.parametrize("kw", [{}, {"patch_enabled": 0}, {"particle_weight": 0.6, "bend_strength": 9.0},
                                {"entry_point": (0.0, 1.0, 0.0), "patch_enabled": 0},
                                {"intensity_falloff": 0.02, "spread_angle": 1.2}])
def test_texture_matches_oracle(sbs, orc, br, kw):
    p = br.BranchedFlowParams.default()
    p.num_rays = 2048
    for k, v in kw.items():
        if k == "entry_point":
            for i, x in enumerate(v):
                p.entry_point[i] = x
        else:
            setattr(p, k, v)
    th = field(scale=2e4)  # thickness in um-ish units so that the GRIN kick matters
    sc = br.generate_scatterers(p, time=1.5)
    tex0 = np.random.default_rng(0).integers(0, 5000, (p.tex_height, p.tex_width)).astype(np.uint32)
    got = br.branched_flow_step(p, th, sc, tex0, fade=True)
    want = orc.branched_flow(p, th, sc, tex0, fade=True)
    assert np.array_equal(got, want), (int(np.abs(got.astype(np.int64) - want).max()), int((got != want).sum()))
    assert got.sum() > tex0.sum() * 0.85 * 0.9  # the rays deposited


def test_simulator_steps(sbs, br):
    sim = br.BranchedFlowSimulator()
    sim.params.num_rays = 4096
    sim.params.patch_enabled = 0  # the default entry point (u = 0.75) lies outside the default patch
    th = field(scale=2e4)
    t1 = sim.step(th, 0.0).copy()
    t2 = sim.step(th, 0.016)
    assert t1.sum() > 0 and t2.sum() > t1.sum()  # fade x 0.85 plus a new frame of deposits
    assert sim.texture_size() == (512, 256)


def test_bad_arguments(sbs, br):
    p = br.BranchedFlowParams.default()
    with pytest.raises(ValueError):
        br.branched_flow_step(p, field(), np.zeros((10, 4), np.float32), np.zeros((256, 512), np.uint32))
    p.tex_width = 1
    with pytest.raises(sbs.SbsError):
        br.branched_flow_step(p, field(), br.generate_scatterers(br.BranchedFlowParams.default()),
                              np.zeros((256, 1), np.uint32))
