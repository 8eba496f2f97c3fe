"""Foam cluster dynamics on the GPU (sbs_foam_sim_*) against the oracle's restatement of the
reference's O(n^2) loops (foam_dynamics.rs:62-238, foam.rs:322-405).

Bar: bit for bit. The kernel forms each bubble's force sum in the reference's order from a
neighbour list sorted by bubble order (pairs beyond 3 (r_a + r_b) add exact zeros), with the same
f32 operations, so forces, positions, velocities, ids and the connection records are equal as
arrays after any number of steps, merges included. (The merged radius x^(1/3) is rounded once
from double on both sides; CUDA's and glibc's double pow could differ in the last double bit,
which changes the float only for a near-tie, about one merge in 10^8.)"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def fd(sbs):
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


def _same_state(sim, want):
    got = sim.bubbles()
    for k in ("position", "velocity", "radius", "thickness_nm", "ids"):
        np.testing.assert_array_equal(got[k], want[k], err_msg=k)
    c = sim.connections()
    w = want["connections"]
    assert len(c) == len(w) == sim.connection_count()
    for k in w.dtype.names:
        np.testing.assert_array_equal(c[k], w[k], err_msg=k)


def test_default_cluster_reference_tests(fd, orc):
    sim = fd.FoamSimulator.with_default_cluster()
    assert sim.bubble_count() == 5 and sim.connection_count() > 0  # foam.rs:534-579
    assert sim.compute_forces().shape == (5, 3)
    pos, rad = fd.default_cluster()
    want = orc.foam_step(sim.physics, 0.016, 0, pos, rad)
    _same_state(sim, want)
    for k in range(11):  # test_connections_after_physics_step (foam.rs:512-531)
        sim.step(0.016)
    _same_state(sim, orc.foam_step(sim.physics, 0.016, 11, pos, rad))
    sim.reset()  # FoamSimulator::reset: the default cluster again
    np.testing.assert_array_equal(sim.bubbles()["position"], pos)
    assert sim.query_nearby([0.0, 0.0, 0.0], 0.1) == [2, 4, 0, 1, 3]  # cells (-1,0,0), (0,-1,0), (0,0,0)
    # test_repulsion_separates_overlapping_bubbles (foam_dynamics.rs:348-367)
    s2 = fd.FoamSimulator([[0, 0, 0], [0.04, 0, 0]], [0.03, 0.03], physics=_phys(fd, gravity=[0.0, 0.0, 0.0]))
    s2.step(0.001, 100)
    b = s2.bubbles()
    assert np.linalg.norm(b["position"][0] - b["position"][1]) > 0.04


@pytest.mark.parametrize("n,seed", [(300, 0), (2000, 1), (5000, 2)])
def test_forces_match_oracle(fd, orc, n, seed):
    pos, rad = fd.fcc_foam(n, seed=seed)
    g = np.random.default_rng(seed + 10)
    vel = g.normal(0, 0.03, (n, 3)).astype(np.float32)
    th = g.uniform(50, 1500, n).astype(np.float32)
    sim = fd.FoamSimulator(pos, rad, thickness_nm=th)
    sim.set_state(velocity=vel)
    np.testing.assert_array_equal(sim.compute_forces(), orc.foam_forces(sim.physics, pos, rad, velocity=vel,
                                                                        thickness_nm=th))


@pytest.mark.parametrize("dt,steps", [(1e-3, 40), (0.016, 12)])
def test_steps_match_oracle(fd, orc, dt, steps):
    pos, rad = fd.fcc_foam(1200, seed=7)
    sim = fd.FoamSimulator(pos, rad)
    sim.step(dt, steps)
    _same_state(sim, orc.foam_step(sim.physics, dt, steps, pos, rad))
    # one call of k steps equals k calls of one step
    s2 = fd.FoamSimulator(pos, rad)
    for _ in range(steps):
        s2.step(dt)
    np.testing.assert_array_equal(s2.bubbles()["position"], sim.bubbles()["position"])


def test_coalescence_matches_oracle(fd, orc):
    # a cluster shaken hard, with a low Weber threshold: several merges, one per step at most
    pos, rad = fd.fcc_foam(600, seed=11)
    g = np.random.default_rng(12)
    vel = g.normal(0, 0.05, (600, 3)).astype(np.float32)
    p = _phys(fd, coalescence_enabled=1, coalescence_threshold=0.02)
    sim = fd.FoamSimulator(pos, rad, physics=p)
    sim.set_state(velocity=vel)
    want = orc.foam_step(p, 2e-3, 25, pos, rad, velocity=vel)
    sim.step(2e-3, 25)
    assert want["position"].shape[0] < 600  # merges happened
    _same_state(sim, want)


def test_dense_lists(fd, orc):
    """Large bubbles on the same lattice: lists of about 630 candidates, 140 of them above 1024
    (the register sort and the shared-memory sort)."""
    pos, rad = fd.fcc_foam(3000, min_radius=0.028, max_radius=0.036, seed=17)
    sim = fd.FoamSimulator(pos, rad)
    np.testing.assert_array_equal(sim.compute_forces(), orc.foam_forces(sim.physics, pos, rad))
    sim.step(1e-3, 3)
    _same_state(sim, orc.foam_step(sim.physics, 1e-3, 3, pos, rad))


@pytest.mark.parametrize("coalescence", [0, 1])
def test_compression_grows_the_list(fd, orc, coalescence):
    """Bubbles streaming to the centre without damping or forces: neighbour counts rise several
    times over, the list outgrows its storage mid-run and is regrown (the steps after the
    overflowing rebuild are redone from the last completed one); the result stays exact. With
    coalescence the streams also merge, a bubble per step."""
    pos, rad = fd.fcc_foam(1000, spacing=0.05, jitter=0.2, min_radius=0.004, max_radius=0.006, seed=13)
    vel = (-0.1 * pos / np.maximum(np.linalg.norm(pos, axis=1, keepdims=True), 1e-6)).astype(np.float32)
    p = _phys(fd, gravity=[0.0, 0.0, 0.0], damping=1.0, van_der_waals_strength=0.0, repulsion_stiffness=0.0,
              viscosity=0.0, coalescence_enabled=coalescence)
    sim = fd.FoamSimulator(pos, rad, physics=p)
    sim.set_state(velocity=vel)
    sim.step(0.01, 150)
    want = orc.foam_step(p, 0.01, 150, pos, rad, velocity=vel)
    if coalescence:
        assert want["position"].shape[0] < 1000
    _same_state(sim, want)


@pytest.mark.parametrize("n", [40_000, 200_000])
def test_large_cluster_against_subset(fd, orc, n):
    """Large foams (4 lanes per bubble below 131,072 bubbles, 1 above): the forces of sampled
    bubbles against the oracle's reference-order sums for those bubbles (O(n) each), before and
    after 20 steps."""
    pos, rad = fd.fcc_foam(n, seed=21)
    sim = fd.FoamSimulator(pos, rad)
    idx = np.concatenate([np.arange(8), np.random.default_rng(22).integers(0, n, 24), [n - 1]])
    np.testing.assert_array_equal(sim.compute_forces()[idx], orc.foam_forces_subset(sim.physics, pos, rad, idx))
    sim.step(1e-3, 20)
    b = sim.bubbles()
    assert sim.bubble_count() == n and np.abs(np.linalg.norm(b["velocity"], axis=1)).max() <= 0.1 * (1 + 1e-6)
    np.testing.assert_array_equal(sim.compute_forces()[idx],
                                  orc.foam_forces_subset(sim.physics, b["position"], b["radius"], idx,
                                                         velocity=b["velocity"]))


def test_edge_clusters(fd, orc):
    """One bubble; two bubbles on the same centre (the reference's distance < 1e-6 branch: no
    force); far-apart clusters, 1 km and 30 km out (their cells share hash buckets with the
    near ones)."""
    one = fd.FoamSimulator([[0.1, 0.2, 0.3]], [0.02])
    one.step(1e-3, 5)
    _same_state(one, orc.foam_step(one.physics, 1e-3, 5, [[0.1, 0.2, 0.3]], [0.02]))
    same = fd.FoamSimulator([[0, 0, 0], [0, 0, 0], [0.03, 0, 0]], [0.02, 0.02, 0.02])
    np.testing.assert_array_equal(same.compute_forces(),
                                  orc.foam_forces(same.physics, [[0, 0, 0], [0, 0, 0], [0.03, 0, 0]], [0.02] * 3))
    a, ra = fd.fcc_foam(300, seed=31)
    b, rb = fd.fcc_foam(200, seed=32)
    c, rc = fd.fcc_foam(100, seed=33)
    pos = np.concatenate([a, b + np.float32([1000.0, 0, 0]), c + np.float32([-3e4, 2e4, 5.0])]).astype(np.float32)
    rad = np.concatenate([ra, rb, rc])
    g = np.random.default_rng(34)
    order = g.permutation(pos.shape[0])  # the clusters interleaved in bubble order
    pos, rad = pos[order], rad[order]
    sim = fd.FoamSimulator(pos, rad)
    np.testing.assert_array_equal(sim.compute_forces(), orc.foam_forces(sim.physics, pos, rad))
    sim.step(2e-3, 15)
    _same_state(sim, orc.foam_step(sim.physics, 2e-3, 15, pos, rad))


def test_couple_thickness(fd, sbs):
    n = 6
    res = np.array([32, 64, 32, 96, 64, 32], np.uint32)
    radius = np.linspace(0.01, 0.03, n).astype(np.float32)
    batch = sbs.FoamDrainage(res, radius)
    g = np.random.default_rng(5)
    want = []
    for b in range(n):
        nt, npp = int(res[b]), 2 * int(res[b])
        h = (g.uniform(200, 900, (nt, npp)) * 1e-9).astype(np.float32)
        batch.set_thickness(b, h)
        w = np.sin(np.arange(nt) * np.pi / (nt - 1))
        want.append((h.astype(np.float64) * w[:, None]).sum() / (w.sum() * npp) * 1e9)
    pos, rad = fd.fcc_foam(n, seed=1)
    sim = fd.FoamSimulator(pos, rad)
    sim.couple_thickness(batch)
    np.testing.assert_allclose(sim.bubbles()["thickness_nm"], np.array(want), rtol=1e-6)
    with pytest.raises(sbs.SbsError):
        fd.FoamSimulator(*fd.fcc_foam(5)).couple_thickness(batch)


def test_bad_arguments(fd, sbs):
    with pytest.raises(sbs.SbsError):
        fd.FoamSimulator([[0, 0, 0]], [-1.0])
    with pytest.raises(sbs.SbsError):
        fd.FoamSimulator([[0, 0, np.nan]], [0.01])
    sim = fd.FoamSimulator.with_default_cluster()
    with pytest.raises(sbs.SbsError):
        sim.step(float("inf"))
