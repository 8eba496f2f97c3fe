"""Branched flow on the CPU: the library's acos / atan2 / exp against numpy, the scatterer
generation (the library's host code against the oracle's restatement, bit for bit) and the
reference's own tests of generate_scatterers (branched_flow.rs:700-847), the fade pass."""
import math

import numpy as np
import pytest


@pytest.fixture(scope="module")
def br():
    from soap_bubble_simulation_gb300 import branched

    return branched


def test_own_transcendentals_match_numpy(orc):
    xs = np.linspace(-1, 1, 4001)
    e = max(abs(orc.acos_as(x) - math.acos(np.float32(x))) for x in xs)
    assert e < 5e-7, e  # A&S 2e-8 plus the float evaluation (pi - r near x = -1)
    g = np.random.default_rng(0)
    pts = g.normal(size=(4000, 2))
    e = max(abs(orc.atan2_as(y, x) - math.atan2(np.float32(y), np.float32(x))) for y, x in pts)
    assert e < 5e-7, e
    assert orc.atan2_as(-0.0, -1.0) == -orc.atan2_as(0.0, -1.0) and abs(orc.atan2_as(0.0, -1.0) - math.pi) < 3e-7
    xs = np.linspace(-20, 20, 4001)
    e = max(abs(orc.exp_cw(x) / math.exp(np.float32(x)) - 1) for x in xs)
    assert e < 3e-7, e


def _params(br, **kw):
    p = br.BranchedFlowParams.default()
    for k, v in kw.items():
        setattr(p, k, v)
    return p


@pytest.mark.parametrize("patch,time", [(1, 0.0), (0, 0.0), (0, 3.7), (1, 12.5)])
def test_scatterers_library_equals_oracle(orc, br, patch, time):
    p = _params(br, patch_enabled=patch, patch_half_size=0.2)
    np.testing.assert_array_equal(br.generate_scatterers(p, 800, time), orc.branched_scatterers(p, 800, time))


def test_reference_scatterer_properties(br):
    p = _params(br, patch_enabled=0)  # generate_scatterers(..., None): no patch bounds
    assert br.generate_scatterers(p, 100).shape == (100, 4) and br.generate_scatterers(p, 500).shape == (500, 4)
    s = br.generate_scatterers(p, 200)
    assert (s[:, 0] >= 0).all() and (s[:, 0] <= 1).all() and (s[:, 1] >= 0).all() and (s[:, 1] <= 1).all()
    s = br.generate_scatterers(p, 100)
    assert (s[:, 2] > 0).sum() > 20 and (s[:, 2] < 0).sum() > 20
    assert (s[:, 3] > 0).all()
    a, b = br.generate_scatterers(p, 50, 0.0), br.generate_scatterers(p, 50, 1.0)
    assert (np.abs(a[:, :2] - b[:, :2]).max(axis=1) > 0.001).sum() > 0
    pp = _params(br, patch_enabled=1, patch_center_u=0.5, patch_center_v=0.5, patch_half_size=0.2)
    s = br.generate_scatterers(pp, 100)
    assert (s[:, 0] >= 0.2).all() and (s[:, 0] <= 0.8).all() and (s[:, 1] >= 0.2).all() and (s[:, 1] <= 0.8).all()


def test_struct_layouts(br):
    import ctypes

    assert ctypes.sizeof(br.BranchedFlowParams) == 112
    assert br.BranchedFlowParams.num_scatterers.offset == 80 and br.BranchedFlowParams.patch_half_size.offset == 108


def test_fade_and_deposit_budget(orc, br):
    p = _params(br, num_rays=64, num_scatterers=100, patch_enabled=0)
    th = np.full((64, 128), 5e-7, np.float32)
    sc = orc.branched_scatterers(p, 100, 0.0)
    tex0 = np.random.default_rng(1).integers(0, 10000, (256, 512)).astype(np.uint32)
    faded = orc.branched_flow(_params(br, num_rays=0), th, sc, tex0, fade=True)
    np.testing.assert_array_equal(faded, (tex0.astype(np.float32) * np.float32(0.85)).astype(np.uint32))
    tex = orc.branched_flow(p, th, sc, np.zeros((256, 512), np.uint32), fade=False)
    # a ray deposits at most 0.15 * 256 per step (truncation only loses); 400 steps, falloff 0.001
    budget = 64 * sum(0.15 * 256 * 0.999 ** k for k in range(400))
    assert 0.5 * budget < tex.sum() <= budget
