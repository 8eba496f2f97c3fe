"""Batched foam drainage: every bubble of a batch equals the single-bubble GPUDrainageSimulator
bit for bit (same drainage.wgsl arithmetic), for every tile shape and around autotuning."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

RES = [32, 64, 32, 96, 160, 256, 64, 32, 128, 224, 40, 48]


def batch(sbs, res, seed=0, marangoni=False):
    from soap_bubble_simulation_gb300 import synthetic as S

    g = np.random.default_rng(seed)
    rad = g.uniform(0.001, 0.04, len(res)).astype(np.float32)
    params = sbs.DrainageParams(marangoni_enabled=1 if marangoni else 0)
    foam = sbs.FoamDrainage(res, rad, params)
    hs = S.foam_fields(np.asarray(res, dtype=np.uint32), seed=seed)
    cs = [S.surfactant_noise(r, 2 * r, seed=seed + i) for i, r in enumerate(res)]
    for b in range(len(res)):
        foam.set_thickness(b, hs[b])
        foam.set_concentration(b, cs[b])
    return foam, rad, hs, cs


def single(sbs, r, radius, h, c, steps, marangoni):
    sim = sbs.GPUDrainageSimulator(None, 500e-9, 2 * r, r)
    sim.set_bubble_radius(float(radius))
    sim.set_marangoni_enabled(marangoni)
    sim.set_thickness_array(h)
    sim.set_concentration_array(c)
    sim.run(steps)
    return sim.thickness_array(), sim.concentration_array()


@pytest.mark.parametrize("marangoni", [False, True])
def test_foam_bubbles_equal_single_bubble_path(sbs, marangoni):
    foam, rad, hs, cs = batch(sbs, RES, seed=1, marangoni=marangoni)
    foam.run(37)
    for b, r in enumerate(RES):
        h1, c1 = single(sbs, r, rad[b], hs[b], cs[b], 37, marangoni)
        np.testing.assert_array_equal(foam.thickness(b), h1, err_msg=f"bubble {b} (res {r})")
        np.testing.assert_array_equal(foam.concentration(b), c1, err_msg=f"bubble {b} (res {r})")


@pytest.mark.parametrize("k,rb", [(1, 8), (2, 16), (4, 64), (4, 4)])
def test_foam_tile_shapes_agree(sbs, k, rb):
    ref, _, _, _ = batch(sbs, RES, seed=2)
    ref.set_tiles(4, 32)
    ref.run(21)
    foam, _, _, _ = batch(sbs, RES, seed=2)
    foam.set_tiles(k, rb)
    foam.run(10)
    foam.run(11)
    for b in range(len(RES)):
        np.testing.assert_array_equal(foam.thickness(b), ref.thickness(b))


def test_foam_autotune_keeps_fields(sbs):
    ref, _, _, _ = batch(sbs, RES, seed=3)
    ref.run(13)
    foam, _, _, _ = batch(sbs, RES, seed=3)
    k, rb = foam.autotune(trial_steps=8)
    assert k in (2, 4) and rb in (8, 16, 32, 64)
    foam.run(13)
    for b in range(len(RES)):
        np.testing.assert_array_equal(foam.thickness(b), ref.thickness(b))
    assert foam.total_cells() == sum(2 * r * r for r in RES)


def test_foam_rejects_bad_input(sbs):
    with pytest.raises(sbs.SbsError):
        sbs.FoamDrainage([32, 2], [0.01, 0.01])
    with pytest.raises(sbs.SbsError):
        sbs.FoamDrainage([32], [-1.0])
    foam = sbs.FoamDrainage([32], [0.01])
    with pytest.raises(ValueError):
        foam.set_thickness(0, np.zeros((32, 32), np.float32))
