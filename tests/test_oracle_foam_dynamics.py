"""Foam cluster dynamics on the CPU: the oracle's restatement of FoamSimulator / BubbleCluster
(foam_dynamics.rs, foam.rs) against the reference's own unit tests (foam_dynamics.rs:300-368,
foam.rs:426-580), closed forms of its force terms, and the library's host-side pieces (defaults,
struct layouts, the FCC cluster layout)."""
import math

import numpy as np
import pytest

f32 = np.float32


@pytest.fixture(scope="module")
def fd():
    from soap_bubble_simulation_gb300 import foam_dynamics

    return foam_dynamics


def _phys(fd, **kw):
    p = fd.FoamPhysics.default()
    for k, v in kw.items():
        if k == "gravity":
            p.gravity[:] = v
        else:
            setattr(p, k, v)
    return p


def test_defaults_and_layouts(fd):
    import ctypes

    p = fd.FoamPhysics.default()
    assert (p.surface_tension, p.viscosity, p.density) == (f32(0.025), f32(0.001), 1000.0)
    assert list(p.gravity) == [0.0, f32(-9.81), 0.0]
    assert (p.van_der_waals_strength, p.repulsion_stiffness, p.damping) == (f32(0.001), 5.0, f32(0.8))
    assert p.coalescence_enabled == 0 and p.coalescence_threshold == 0.5
    assert ctypes.sizeof(fd.FoamPhysics) == 48 and fd.CONNECTION.itemsize == 40
    pos, rad = fd.default_cluster()
    assert pos.shape == (5, 3) and rad.shape == (5,)


def test_pow15_is_the_rounded_power(orc):
    """The library's x^1.5 (the Hertz term) against the correctly rounded value from float64."""
    g = np.random.default_rng(0)
    xs = np.concatenate([g.uniform(0, 0.06, 200000), 10.0 ** g.uniform(-12, 1, 100000)]).astype(np.float32)
    got = np.array([orc.pow15(x) for x in xs], dtype=np.float32)
    want = (xs.astype(np.float64) ** 1.5).astype(np.float32)
    ulp = np.abs(got.view(np.int32).astype(np.int64) - want.view(np.int32).astype(np.int64))
    assert ulp.max() <= 1 and (ulp == 0).mean() > 0.99999, ((ulp == 0).mean(), ulp.max())


# --- the reference's tests (foam_dynamics.rs:304-367, foam.rs:430-579) -----------------------------
def test_reference_simulator_step_and_forces(orc, fd):
    p = _phys(fd)
    pos, rad = fd.default_cluster()
    assert orc.foam_forces(p, pos, rad).shape == (5, 3)  # test_force_computation
    r = orc.foam_step(p, 0.001, 1, pos, rad)
    assert r["position"].shape[0] == 5  # test_simulation_step: no coalescence
    assert len(orc.foam_step(p, 0.016, 0, pos, rad)["connections"]) > 0  # test_default_cluster_has_connections


def test_reference_buoyancy_reduces_gravity(orc, fd):
    # one bubble at rest: the force is its buoyancy-adjusted gravity alone
    p = _phys(fd)
    f = orc.foam_forces(p, [[0, 0, 0]], [0.025])[0]
    g = np.array([0.0, -1.0, 0.0])
    n = np.linalg.norm(f)
    assert n < 1e-6 or abs(np.dot(f / n, g)) > 0.99


def test_reference_repulsion_separates(orc, fd):
    p = _phys(fd, gravity=[0.0, 0.0, 0.0])
    r = orc.foam_step(p, 0.001, 100, [[0, 0, 0], [0.04, 0, 0]], [0.03, 0.03])
    assert np.linalg.norm(r["position"][0] - r["position"][1]) > 0.04


def test_reference_merge_conserves_volume(orc, fd):
    # two overlapping bubbles approaching each other: with coalescence on and a zero Weber
    # threshold the first step merges them (merge_bubbles, foam.rs:369-405)
    p = _phys(fd, gravity=[0.0, 0.0, 0.0], coalescence_enabled=1, coalescence_threshold=0.0)
    vol = 2 * (f32(4.0) / f32(3.0)) * f32(math.pi) * f32(0.5) ** 3
    r = orc.foam_step(p, 1e-6, 1, [[0, 0, 0], [0.8, 0, 0]], [0.5, 0.5], velocity=[[0.01, 0, 0], [-0.01, 0, 0]])
    assert r["position"].shape[0] == 1 and r["ids"][0] == 2 and r["next_id"] == 3
    v = (4.0 / 3.0) * math.pi * float(r["radius"][0]) ** 3
    assert abs(v - vol) < 1e-6
    assert len(r["connections"]) == 0  # the merged pair's connection is dropped (remove_bubble's retain)


def test_reference_connection_curvature(orc, fd):
    p = _phys(fd)
    c = orc.foam_step(p, 0.0, 0, [[0, 0, 0], [0.05, 0, 0]], [0.03, 0.02])["connections"]
    assert len(c) == 1 and np.isfinite(c["wall_curvature_radius"][0])
    # Young-Laplace: R_wall = 2 gamma / (4 gamma / r_a - 4 gamma / r_b) < 0 toward the smaller bubble
    want = 2 * 0.025 / (4 * 0.025 / 0.03 - 4 * 0.025 / 0.02)
    assert abs(c["wall_curvature_radius"][0] - want) < 1e-6 and c["wall_curvature_radius"][0] < 0
    eq = orc.foam_step(p, 0.0, 0, [[0, 0, 0], [0.05, 0, 0]], [0.03, 0.03])["connections"]
    assert np.isinf(eq["wall_curvature_radius"][0])  # flat wall between equal bubbles
    np.testing.assert_allclose(c["contact_point"][0], [0.05 * 0.6, 0, 0], atol=1e-8)
    np.testing.assert_array_equal(c["contact_normal"][0], [1, 0, 0])
    assert c["wall_thickness_nm"][0] == f32(400.0)


# --- closed forms of the force terms -------------------------------------------------------------
def test_force_terms_closed_form(orc, fd):
    p = _phys(fd, gravity=[0.0, 0.0, 0.0])
    ra, rb = 0.02, 0.03
    s = ra + rb
    for d, kind in ((2.0 * s, "vdw"), (1.1 * s, "vdw+adhesion"), (0.9 * s, "repulsion+adhesion"),
                    (0.97 * s, "repulsion+adhesion"), (3.5 * s, "none")):
        f = orc.foam_forces(p, [[0, 0, 0], [d, 0, 0]], [ra, rb]).astype(np.float64)
        d, ra_, rb_ = float(f32(d)), float(f32(ra)), float(f32(rb))
        s_ = ra_ + rb_
        terms = []
        if s_ < d < 3 * s_:
            terms.append(0.001 * ra_ * rb_ / d ** 2)
        if d < s_:
            terms.append(-5.0 * (s_ - d) ** 1.5)
        if 0.95 * s_ < d < 1.2 * s_:
            terms.append(2.0 * (1.2 * s_ - d))
        want = sum(terms)
        tol = 1e-6 * sum(abs(t) for t in terms) + 1e-12  # f32 rounding of each term
        assert abs(f[0, 0] - want) <= tol, (kind, f[0, 0], want)
        assert f[1, 0] == -f[0, 0] and f[0, 1] == 0 and f[0, 2] == 0
    # drag only: -6 pi eta r v
    f = orc.foam_forces(p, [[0, 0, 0]], [0.02], velocity=[[0.05, 0, 0]])[0]
    want = -6 * math.pi * 0.001 * 0.02 * 0.05
    assert abs(f[0] - want) < 1e-6 * abs(want)


def test_subset_forces_equal_the_full_loop(orc, fd):
    pos, rad = fd.fcc_foam(1500, seed=3)
    g = np.random.default_rng(4)
    vel = g.normal(0, 0.03, (1500, 3)).astype(np.float32)
    th = g.uniform(100, 900, 1500).astype(np.float32)
    p = _phys(fd)
    full = orc.foam_forces(p, pos, rad, velocity=vel, thickness_nm=th)
    idx = np.array([0, 1, 17, 700, 1498, 1499])
    np.testing.assert_array_equal(orc.foam_forces_subset(p, pos, rad, idx, velocity=vel, thickness_nm=th), full[idx])


def test_far_pairs_contribute_nothing(orc, fd):
    """A cluster split in two far halves: each half's forces equal those of the half alone, the
    premise of the neighbour-list evaluation (pairs beyond 3 (r_a + r_b) add exact zeros)."""
    pos, rad = fd.fcc_foam(400, seed=5)
    far = pos.copy()
    far[200:, 0] += 10.0
    p = _phys(fd)
    f = orc.foam_forces(p, far, rad)
    np.testing.assert_array_equal(f[:200], orc.foam_forces(p, far[:200], rad[:200]))
    np.testing.assert_array_equal(f[200:], orc.foam_forces(p, far[200:], rad[200:]))


def test_fcc_layout(fd):
    pos, rad = fd.fcc_foam(500, jitter=0.0)
    n = 5  # ceil(cbrt(500 / 4))
    assert pos.shape == (500, 3) and rad.min() >= 0.015 and rad.max() <= 0.03
    np.testing.assert_allclose(pos[0], [-(n - 1) * 0.05 / 2] * 3, atol=1e-7)
    np.testing.assert_allclose(pos[1] - pos[0], [0.025, 0.025, 0.0], atol=1e-7)
    assert len({tuple(np.round(q, 6)) for q in pos}) == 500


def test_no_gpu_is_an_error_not_a_fallback(fd):
    """Without a GPU the simulator refuses to start (no CPU path); bad arguments are rejected
    before the device is looked at."""
    import ctypes

    from soap_bubble_simulation_gb300 import _native as N

    with pytest.raises(N.SbsError) as bad:
        fd.FoamSimulator([[0.0, 0.0, 0.0]], [-1.0])
    assert bad.value.code == N.SBS_E_INVALID
    n = ctypes.c_int(-1)
    if N.lib().sbs_device_count(ctypes.byref(n)) == 0 and n.value > 0:
        pytest.skip("a GPU is visible here")
    with pytest.raises(N.SbsError) as e:
        fd.FoamSimulator([[0.0, 0.0, 0.0]], [0.01])
    assert e.value.code == N.SBS_E_CUDA


def test_reference_spatial_hash(fd):
    """foam.rs:470-480 (test_spatial_hash), and the query order of SpatialHash::query."""
    h = fd.SpatialHash(1.0)
    h.insert(0, [0.0, 0.0, 0.0])
    h.insert(1, [0.5, 0.0, 0.0])
    h.insert(2, [5.0, 0.0, 0.0])
    near = h.query([0.0, 0.0, 0.0], 1.0)
    assert 0 in near and 1 in near and 2 not in near
    h.insert(3, [-0.5, -0.5, -0.5])  # cell (-1, -1, -1): the first offset walked
    assert h.query([0.0, 0.0, 0.0], 1.0) == [3, 0, 1]
    h.rebuild([7, 8], [[0.2, 0.2, 0.2], [3.0, 3.0, 3.0]])
    assert h.query([0.0, 0.0, 0.0], 0.5) == [7]


def test_argument_validation_before_device(fd):
    """The C ABI rejects bad arguments with SBS_E_INVALID before it looks for a device."""
    import ctypes

    from soap_bubble_simulation_gb300 import _native as N

    L = N.lib()
    p = fd.FoamPhysics.default()
    pp = ctypes.cast(ctypes.byref(p), ctypes.c_void_p)
    pos = np.zeros((2, 3), np.float32)
    rad = np.full(2, 0.01, np.float32)
    h = ctypes.c_void_p()
    assert L.sbs_foam_sim_create(0, N.ptr(pos), N.ptr(rad), None, pp, ctypes.byref(h)) == N.SBS_E_INVALID
    assert L.sbs_foam_sim_create(2, None, N.ptr(rad), None, pp, ctypes.byref(h)) == N.SBS_E_INVALID
    assert L.sbs_foam_sim_create(2, N.ptr(pos), N.ptr(rad), None, None, ctypes.byref(h)) == N.SBS_E_INVALID
    bad = fd.FoamPhysics.default()
    bad.damping = float("nan")
    assert L.sbs_foam_sim_create(2, N.ptr(pos), N.ptr(rad), None, ctypes.cast(ctypes.byref(bad), ctypes.c_void_p),
                                 ctypes.byref(h)) == N.SBS_E_INVALID
    assert b"finite" in L.sbs_last_error()
    thick = np.array([500.0, np.inf], np.float32)
    assert L.sbs_foam_sim_create(2, N.ptr(pos), N.ptr(rad), N.ptr(thick), pp, ctypes.byref(h)) == N.SBS_E_INVALID
    assert not h
    for fn, args in (("sbs_foam_sim_step", (None, 1e-3, 1)), ("sbs_foam_sim_counts", (None, None, None)),
                     ("sbs_foam_sim_forces", (None, None, N.MEM_HOST)),
                     ("sbs_foam_sim_couple_thickness", (None, None))):
        assert getattr(L, fn)(*args) == N.SBS_E_INVALID, fn
    assert L.sbs_foam_sim_destroy(None) == 0
    out = fd.FoamPhysics()
    assert L.sbs_foam_physics_default(None) == N.SBS_E_INVALID
    assert L.sbs_foam_physics_default(ctypes.cast(ctypes.byref(out), ctypes.c_void_p)) == 0


def test_set_physics_keeps_the_old_values_on_error(fd):
    """set_physics builds the new values on a copy: a rejected update leaves the simulator's physics
    as they were (exercised here without a device through the library's argument check)."""
    from soap_bubble_simulation_gb300 import _native as N

    sim = fd.FoamSimulator.__new__(fd.FoamSimulator)  # no device: a handle-less simulator
    sim.physics = fd.FoamPhysics.default()
    sim._h = None
    with pytest.raises(N.SbsError):
        sim.set_physics(damping=float("nan"))
    assert sim.physics.damping == np.float32(0.8)
