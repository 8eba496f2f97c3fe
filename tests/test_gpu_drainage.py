"""GPU parity of the drainage kernels through the C ABI (libsbs.so) against the oracle.

Bars:
  * bit-exact against the kernel-order oracle (same f32 arithmetic), both semantics, all sizes;
  * CPU semantics vs the f64 restatement of drainage.rs: relative L-inf <= 1e-5 per step and,
    after 1000 steps of config 0, <= 1e-4 (plain f32) / <= 1e-8 (compensated f32x2);
  * WGSL semantics vs the drainage.wgsl operation order: <= 1e-5 per pass, <= 1e-4 after 1000;
  * FP64 film volume within 1e-12 relative of the oracle's sum.
"""
import ctypes
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def rel_linf(a, b):
    return float(np.max(np.abs(np.asarray(a, np.float64) - b)) / np.max(np.abs(b)))


def make_sim(sbs, res, precision="f32x2"):
    cfg = sbs.SimulationConfig()
    cfg.resolution = res
    c = cfg.to_c()
    h = ctypes.c_void_p()
    prec = sbs._native.DRAIN_F32X2 if precision == "f32x2" else sbs._native.DRAIN_F32
    sbs._native.call("sbs_drainage_create_ex", ctypes.byref(c), prec, ctypes.byref(h))
    sim = sbs.DrainageSimulator.__new__(sbs.DrainageSimulator)
    sbs.drainage._Handle.__init__(sim)
    sim._h = h
    sim._config = cfg
    return sim


def field64(sbs, sim):
    nt, np_ = sim.grid()
    out = np.empty(nt * np_, dtype=np.float64)
    sbs._native.call("sbs_drainage_get_thickness_field_f64", sim.handle, sbs._native.dptr(out), out.size)
    return out.reshape(nt, np_)


def set64(sbs, sim, h):
    a = np.ascontiguousarray(h, dtype=np.float64)
    sbs._native.call("sbs_drainage_set_thickness_f64", sim.handle, sbs._native.dptr(a), a.size)


ORC_PREC = {"f32": "f32k", "f32x2": "f32x2"}


# --------------------------------------------------------------------------------------------
# CPU semantics (DrainageSimulator)
# --------------------------------------------------------------------------------------------
@pytest.mark.parametrize("precision", ["f32x2", "f32"])
@pytest.mark.parametrize("res", [3, 8, 33, 64, 130])
def test_cpu_semantics_bit_exact(sbs, orc, precision, res):
    """Single steps and graph-replayed chunks, TFE fronts active (dt 0.01 s: first spawn at step
    50), odd and non-multiple-of-4 widths; every cell equal to the kernel-order oracle."""
    from soap_bubble_simulation_gb300 import synthetic

    h0 = synthetic.bubble_c0(res, seed=res)
    if precision == "f32":
        h0 = h0.astype(np.float32).astype(np.float64)
    sim = make_sim(sbs, res, precision)
    set64(sbs, sim, h0)
    ref = orc.CpuSim(resolution=res, precision=ORC_PREC[precision])
    ref.set_field(h0)
    for _ in range(10):
        sim.step(0.01)
        ref.step(0.01)
    np.testing.assert_array_equal(field64(sbs, sim), ref.field())
    sim.step_n(0.01, 190)
    ref.step_n(0.01, 190)
    got, want = field64(sbs, sim), ref.field()
    assert sim.active_tfe_count() == ref.active_tfe_count()
    assert sim.current_time() == ref.current_time()
    if not np.array_equal(got, want):
        bad = np.argwhere(got != want)
        pytest.fail(f"{len(bad)} cells differ, first {bad[:5].tolist()}, "
                    f"max rel {rel_linf(got, want):.3e}")
    if res >= 33:
        assert sim.active_tfe_count() >= 1
        assert (got < h0 * 0.99999).any()  # fronts thinned something


def set_cpu_blocking(sbs, sim, k):
    sbs._native.call("sbs_drainage_set_time_blocking", sim.handle, k)


def cpu_blocking(sbs, sim):
    out = ctypes.c_int()
    sbs._native.call("sbs_drainage_time_blocking", sim.handle, ctypes.byref(out))
    return out.value


@pytest.mark.parametrize("precision", ["f32x2", "f32"])
@pytest.mark.parametrize("res", [10, 12, 64, 130, 256])
def test_cpu_time_blocking_bit_identical(sbs, orc, precision, res):
    """K = 1..4 steps per launch (the blocked kernel's polar strips form each step's ring means
    as exact integer sums across their blocks): the same bits as single steps and as the
    kernel-order oracle, with fronts active (first spawn at step 50), a frozen critical patch,
    volume checks and chunk ends at every K."""
    from soap_bubble_simulation_gb300 import synthetic

    h0 = synthetic.bubble_c0(res, seed=res + 1)
    h0[res // 3, : res // 2] = 5e-9  # below the 10 nm critical thickness: frozen
    if precision == "f32":
        h0 = h0.astype(np.float32).astype(np.float64)
    results = []
    for k in (1, 2, 3, 4):
        sim = make_sim(sbs, res, precision)
        assert cpu_blocking(sbs, sim) == (3 if precision == "f32x2" else 4)  # the defaults
        set_cpu_blocking(sbs, sim, k)
        assert cpu_blocking(sbs, sim) == k
        set64(sbs, sim, h0)
        sim.step_n(0.01, 23)
        vols = sim.run_checked(0.01, 60, 20)
        for _ in range(3):
            sim.step(0.01)
        results.append((field64(sbs, sim), vols, sim.active_tfe_count()))
        sim.close()
    for f, v, n in results[1:]:
        np.testing.assert_array_equal(f, results[0][0])
        np.testing.assert_allclose(v, results[0][1], rtol=1e-12)
        assert n == results[0][2]
    ref = orc.CpuSim(resolution=res, precision=ORC_PREC[precision])
    ref.set_field(h0)
    ref.step_n(0.01, 86)
    np.testing.assert_array_equal(results[0][0], ref.field())
    assert results[0][2] == ref.active_tfe_count() >= 1


@pytest.mark.parametrize("precision", ["f32x2", "f32"])
@pytest.mark.parametrize("res", [1024, 1500])
def test_cpu_single_steps_many_column_blocks(sbs, orc, precision, res):
    """Single steps (K = 1) on grids of 2048 and 3000 columns (many column blocks, the last one
    partly filled: 3000 = 5 x 512 + 440), the phi wrap at both ends, fronts active from step 50
    (dt 0.01 s), volume checks: every cell equal to the kernel-order oracle."""
    from soap_bubble_simulation_gb300 import synthetic

    h0 = synthetic.smooth_modes(res, 2 * res, seed=res)
    if precision == "f32":
        h0 = h0.astype(np.float32).astype(np.float64)
    sim = make_sim(sbs, res, precision)
    set_cpu_blocking(sbs, sim, 1)
    set64(sbs, sim, h0)
    sim.step_n(0.01, 47)
    vols = sim.run_checked(0.01, 16, 8)
    ref = orc.CpuSim(resolution=res, precision=ORC_PREC[precision], threads=0)
    ref.set_field(h0)
    ref.step_n(0.01, 55)
    v0 = orc.film_volume(ref.field(), 0.025)
    ref.step_n(0.01, 8)
    got, want = field64(sbs, sim), ref.field()
    assert sim.active_tfe_count() == ref.active_tfe_count() >= 1
    np.testing.assert_array_equal(got, want)
    assert vols[0] == pytest.approx(v0, rel=1e-12)
    assert vols[1] == pytest.approx(orc.film_volume(want, 0.025), rel=1e-12)


def test_cpu_time_blocking_needs_even_resolution(sbs):
    sim = make_sim(sbs, 33)  # 66 columns: not a multiple of 4
    assert cpu_blocking(sbs, sim) == 1
    with pytest.raises(sbs.SbsError, match="even resolution"):
        set_cpu_blocking(sbs, sim, 4)
    set_cpu_blocking(sbs, sim, 1)
    sim.step_n(0.001, 5)
    small = make_sim(sbs, 4)  # fewer than 2 (K + 1) rows for any K
    assert cpu_blocking(sbs, small) == 1
    with pytest.raises(sbs.SbsError):
        set_cpu_blocking(sbs, small, 4)


def test_step_n_equals_repeated_steps(sbs):
    from soap_bubble_simulation_gb300 import synthetic

    h0 = synthetic.bubble_c0(64, seed=3)
    a, b = make_sim(sbs, 64), make_sim(sbs, 64)
    set64(sbs, a, h0)
    set64(sbs, b, h0)
    a.step_n(0.002, 333)
    for _ in range(333):
        b.step(0.002)
    np.testing.assert_array_equal(field64(sbs, a), field64(sbs, b))
    assert a.current_time() == b.current_time()


@pytest.mark.parametrize("precision,tol", [("f32", 1e-4), ("f32x2", 1e-8)])
def test_c0_1000_steps_vs_f64_reference(sbs, orc, precision, tol):
    """Config 0: resolution 128, h = 500 nm (1 + 0.05 U[-1,1]) seed 0, defaults, dt 1e-3,
    1000 steps, TFE on. Relative L-inf against the f64 restatement of drainage.rs."""
    from soap_bubble_simulation_gb300 import synthetic

    h0 = synthetic.bubble_c0(128, seed=0).astype(np.float32).astype(np.float64)
    sim = make_sim(sbs, 128, precision)
    set64(sbs, sim, h0)
    ref = orc.CpuSim(resolution=128, precision="f64", threads=0)
    ref.set_field(h0)
    # per-step bar over the first steps, from the same input each time
    for k in range(5):
        ref_step = orc.CpuSim(resolution=128, precision="f64")
        ref_step.set_field(field64(sbs, sim))
        sim.step(0.001)
        ref_step.step(0.001)
        assert rel_linf(field64(sbs, sim), ref_step.field()) <= 1e-5
    ref.step_n(0.001, 5)
    sim.step_n(0.001, 995)
    ref.step_n(0.001, 995)
    err = rel_linf(field64(sbs, sim), ref.field())
    assert err <= tol, err
    assert sim.active_tfe_count() == ref.active_tfe_count() >= 1


# --- the reference's drainage.rs unit tests on the GPU path (drainage.rs:636-719) ------------
def test_reference_unit_tests_on_gpu(sbs):
    cfg = sbs.SimulationConfig.default()
    sim = sbs.DrainageSimulator(cfg)
    assert abs(sim.current_time()) < 1e-300 and not sim.has_critical_region()
    assert abs(sim.get_thickness(0.5, 1.0) - sim.get_thickness(1.5, 3.0)) < 1e-15
    assert abs(sim.get_thickness(1.0, 0.0) - sim.get_thickness(1.0, 2 * math.pi)) < 1e-12
    before = sim.get_thickness(0.1, 0.0)
    sim.step(cfg.dt)
    assert abs(sim.current_time() - 0.001) < np.finfo(float).eps
    for _ in range(99):
        sim.step(cfg.dt)
    assert sim.get_thickness(0.1, 0.0) < before
    sim.reset(600e-9)
    assert sim.current_time() == 0.0
    assert abs(sim.get_thickness(0.5, 0.5) - 600e-9) < 1e-15
    assert sim.critical_thickness() == pytest.approx(10e-9)
    f = sim.thickness_field()
    assert f.num_theta() == 128 and f.num_phi() == 256


def test_query_batch_matches_oracle(sbs, orc):
    from soap_bubble_simulation_gb300 import synthetic

    h0 = synthetic.bubble_c0(48, seed=9)
    sim = make_sim(sbs, 48)
    set64(sbs, sim, h0)
    ref = orc.CpuSim(resolution=48, precision="f32x2")
    ref.set_field(h0)
    sim.step_n(0.001, 20)
    ref.step_n(0.001, 20)
    g = np.random.default_rng(1)
    th = np.concatenate([g.uniform(-0.5, math.pi + 0.5, 500), [0.0, math.pi, 1.0, 1.0]])
    ph = np.concatenate([g.uniform(-10, 10, 500), [0.0, 2 * math.pi, -2 * math.pi, 4 * math.pi - 1e-12]])
    got = sim.get_thickness_batch(th, ph)
    want = np.array([ref.get_thickness(a, b) for a, b in zip(th, ph)])
    np.testing.assert_array_equal(got, want)


def test_volume_checks_match_oracle(sbs, orc):
    from soap_bubble_simulation_gb300 import synthetic

    h0 = synthetic.bubble_c0(96, seed=4)
    sim = make_sim(sbs, 96)
    set64(sbs, sim, h0)
    ref = orc.CpuSim(resolution=96, precision="f32x2")
    ref.set_field(h0)
    vols = sim.run_checked(0.01, 300, 100)
    assert vols.shape == (3,)
    for k in range(3):
        ref.step_n(0.01, 100)
        want = orc.film_volume(ref.field(), 0.025)
        assert vols[k] == pytest.approx(want, rel=1e-12)
    np.testing.assert_array_equal(field64(sbs, sim), ref.field())
    assert sim.film_volume() == pytest.approx(orc.film_volume(ref.field(), 0.025), rel=1e-12)
    mn, mx = sim.min_max()
    assert mn == ref.min_thickness() and mx == ref.max_thickness()


def test_marginal_regeneration_controls(sbs, orc):
    sim = make_sim(sbs, 64)
    ref = orc.CpuSim(resolution=64, precision="f32x2")
    sim.set_tfe_thickness_ratio(0.2)
    assert sim.tfe_thickness_ratio() == 0.5
    sim.set_tfe_thickness_ratio(0.9)
    ref.set_tfe_thickness_ratio(0.9)
    assert sim.marginal_regeneration_enabled()
    sim.step_n(0.01, 120)
    ref.step_n(0.01, 120)
    assert sim.active_tfe_count() == ref.active_tfe_count() >= 1
    np.testing.assert_array_equal(field64(sbs, sim), ref.field())
    sim.set_marginal_regeneration(False)
    ref.set_marginal_regeneration(False)
    assert sim.active_tfe_count() == 0 and not sim.marginal_regeneration_enabled()
    sim.step_n(0.01, 50)
    ref.step_n(0.01, 50)
    np.testing.assert_array_equal(field64(sbs, sim), ref.field())


def test_critical_cells_frozen_and_detected(sbs):
    h0 = np.full((32, 64), 500e-9)
    h0[10, 5] = 5e-9
    sim = make_sim(sbs, 32)
    set64(sbs, sim, h0)
    assert sim.has_critical_region()
    sim.step_n(0.001, 10)
    # frozen at its stored value: 5 nm as a hi + lo f32 pair
    hi = np.float32(5e-9)
    assert field64(sbs, sim)[10, 5] == float(hi) + float(np.float32(5e-9 - float(hi)))


def test_errors_are_reported(sbs):
    with pytest.raises(sbs.SbsError):
        make_sim(sbs, 2)
    sim = make_sim(sbs, 16)
    with pytest.raises(ValueError):
        sim.set_thickness_array(np.zeros((15, 32), np.float32))
    short = np.zeros(15 * 32, np.float32)
    with pytest.raises(sbs.SbsError, match="expected 16 x 32"):
        sbs._native.call("sbs_drainage_set_thickness", sim.handle, sbs._native.ptr(short), short.size,
                         sbs._native.MEM_HOST)
    with pytest.raises(sbs.SbsError):
        sim.step(float("nan"))
    with pytest.raises(sbs.SbsError, match="WGSL"):
        sbs._native.call("sbs_gpu_drainage_run", sim.handle, 1)
    g = sbs.GPUDrainageSimulator(None, 500e-9, 16, 8)
    with pytest.raises(sbs.SbsError, match="CPU"):
        sbs._native.call("sbs_drainage_step", g.handle, 0.001)
    with pytest.raises(sbs.SbsError):
        sbs.GPUDrainageSimulator(None, 500e-9, 2, 8)


def test_film_volume_device_stateless(sbs, orc):
    from soap_bubble_simulation_gb300 import synthetic

    sim = sbs.GPUDrainageSimulator(None, 500e-9, 128, 64)
    h = synthetic.smooth_modes(64, 128).astype(np.float32)
    sim.set_thickness_array(h)
    d = sim.current_thickness_buffer()
    v = sbs.film_volume_device(d.ptr, 64, 128, d.pitch, 0.025)
    assert v == pytest.approx(orc.film_volume(h, 0.025), rel=1e-12)


# --------------------------------------------------------------------------------------------
# WGSL semantics (GPUDrainageSimulator)
# --------------------------------------------------------------------------------------------
@pytest.mark.parametrize("W,H", [(128, 64), (130, 33), (3, 3), (5, 7), (512, 200)])
@pytest.mark.parametrize("marangoni", [0, 1])
def test_wgsl_semantics_bit_exact(sbs, orc, W, H, marangoni):
    from soap_bubble_simulation_gb300 import synthetic

    h = synthetic.smooth_modes(H, W, seed=W + H).astype(np.float32)
    h[H // 2, W // 2] = 20e-9  # below the 30 nm critical thickness: copied
    c = synthetic.surfactant_noise(H, W, seed=7)
    sim = sbs.GPUDrainageSimulator(None, 500e-9, W, H)
    sim.set_thickness_array(h)
    sim.set_concentration_array(c)
    if marangoni:
        sim.set_marangoni_enabled(True)
    sim.run(37)
    p = orc.wgsl_params(grid_width=W, grid_height=H, marangoni_enabled=marangoni)
    hk, ck = orc.wgsl_run(p, h, c, 37, "kernel")
    np.testing.assert_array_equal(sim.thickness_array(), hk)
    np.testing.assert_array_equal(sim.concentration_array(), ck)


@pytest.mark.parametrize("marangoni", [0, 1])
def test_wgsl_semantics_vs_wgsl_operation_order(sbs, orc, marangoni):
    from soap_bubble_simulation_gb300 import synthetic

    W, H = 128, 64
    h = synthetic.smooth_modes(H, W).astype(np.float32)
    c = synthetic.surfactant_noise(H, W)
    sim = sbs.GPUDrainageSimulator(None, 500e-9, W, H)
    sim.set_thickness_array(h)
    sim.set_concentration_array(c)
    sim.set_marangoni_enabled(bool(marangoni))
    p = orc.wgsl_params(marangoni_enabled=marangoni)
    sim.run(1)
    h1, c1 = orc.wgsl_run(p, h, c, 1, "wgsl")
    assert rel_linf(sim.thickness_array(), h1) <= 1e-5
    assert np.max(np.abs(sim.concentration_array() - c1)) <= 1e-5
    sim.run(999)
    hN, cN = orc.wgsl_run(p, h, c, 1000, "wgsl")
    assert rel_linf(sim.thickness_array(), hN) <= 1e-4
    assert np.max(np.abs(sim.concentration_array() - cN)) <= 1e-4


def test_wgsl_step_clock_and_enable(sbs):
    sim = sbs.GPUDrainageSimulator(None, 500e-9, 128, 64)
    before = sim.thickness_array()
    sim.step(1.0 / 60.0)  # disabled by default (gpu_drainage.rs:339-341)
    np.testing.assert_array_equal(sim.thickness_array(), before)
    assert sim.current_time() == 0.0
    sim.enabled = True
    sim.step(1.0 / 60.0)
    step_dt = np.float32(np.float32(1.0 / 60.0) * np.float32(100.0)) / np.float32(10)
    assert sim.current_time() == pytest.approx(10 * float(step_dt), rel=1e-12)
    assert sim.grid_size() == (128, 64)
    p = sim.params()
    assert p.grid_width == 128 and p.dt == pytest.approx(0.001)


def test_wgsl_buffers_and_reset(sbs, orc):
    """current_buffer() is the last pass's input (gpu_drainage.rs:473-479): its film volume equals
    the field before the pass; current_thickness_buffer() holds the output."""
    from soap_bubble_simulation_gb300 import synthetic

    h = synthetic.smooth_modes(64, 128).astype(np.float32)
    sim = sbs.GPUDrainageSimulator(None, 500e-9, 128, 64)
    sim.set_thickness_array(h)
    sim.run(3)
    prev = orc.wgsl_run(orc.wgsl_params(), h, np.full_like(h, 0.5), 2, "kernel")[0]
    cur = sim.thickness_array()
    stale, new = sim.current_buffer(), sim.current_thickness_buffer()
    assert stale.ptr != new.ptr
    v_stale = sbs.film_volume_device(stale.ptr, 64, 128, stale.pitch, 0.025)
    v_new = sbs.film_volume_device(new.ptr, 64, 128, new.pitch, 0.025)
    assert v_stale == pytest.approx(orc.film_volume(prev, 0.025), rel=1e-12)
    assert v_new == pytest.approx(orc.film_volume(cur, 0.025), rel=1e-12)
    sim.reset(400e-9)
    np.testing.assert_array_equal(sim.thickness_array(), np.float32(400e-9))
    np.testing.assert_array_equal(sim.concentration_array(), np.float32(0.5))
    assert sim.current_time() == 0.0


def test_wgsl_params_setters(sbs, orc):
    from soap_bubble_simulation_gb300 import synthetic

    W, H = 128, 64
    h = synthetic.smooth_modes(H, W).astype(np.float32)
    c = synthetic.surfactant_noise(H, W)
    sim = sbs.GPUDrainageSimulator(None, 500e-9, W, H)
    sim.set_thickness_array(h)
    sim.set_concentration_array(c)
    sim.set_dt(0.002)
    sim.set_physics(0.002, 1100.0, 9.0, 2e-9)
    sim.set_bubble_radius(0.01)
    sim.set_marangoni_params(0.07, 0.05, 3e-9, 0.02)
    sim.set_marangoni_enabled(True)
    sim.run(25)
    p = orc.wgsl_params(dt=0.002, viscosity=0.002, density=1100.0, gravity=9.0, diffusion_coeff=2e-9,
                        bubble_radius=0.01, gamma_air=0.07, gamma_reduction=0.05, surfactant_diffusion=3e-9,
                        marangoni_coeff=0.02, marangoni_enabled=1)
    hk, ck = orc.wgsl_run(p, h, c, 25, "kernel")
    np.testing.assert_array_equal(sim.thickness_array(), hk)
    np.testing.assert_array_equal(sim.concentration_array(), ck)


def test_wgsl_volume_checks(sbs, orc):
    from soap_bubble_simulation_gb300 import synthetic

    W, H = 256, 128
    h = synthetic.smooth_modes(H, W).astype(np.float32)
    c = synthetic.surfactant_noise(H, W)
    sim = sbs.GPUDrainageSimulator(None, 500e-9, W, H)
    sim.set_thickness_array(h)
    sim.set_concentration_array(c)
    vols = sim.run_checked(0.0, 200, 50)
    p = orc.wgsl_params(grid_width=W, grid_height=H)
    cur_h, cur_c = h, c
    for k in range(4):
        cur_h, cur_c = orc.wgsl_run(p, cur_h, cur_c, 50, "kernel")
        assert vols[k] == pytest.approx(orc.film_volume(cur_h, 0.025), rel=1e-12)


# --------------------------------------------------------------------------------------------
# Temporal blocking (several WGSL steps per launch) must not change a single bit
# --------------------------------------------------------------------------------------------
def set_blocking(sbs, sim, k):
    sbs._native.call("sbs_gpu_drainage_set_time_blocking", sim.handle, k)


@pytest.mark.parametrize("W,H", [(4096, 300), (512, 200), (8, 5), (132, 40), (248, 9)])
@pytest.mark.parametrize("marangoni", [0, 1])
def test_time_blocking_bit_identical(sbs, orc, W, H, marangoni):
    from soap_bubble_simulation_gb300 import synthetic

    h = synthetic.smooth_modes(H, W, seed=W * 7 + H).astype(np.float32)
    h[H // 3, : W // 5] = 25e-9  # a patch below the critical thickness
    c = synthetic.surfactant_noise(H, W, seed=H)
    results = []
    for k in (1, 2, 3, 4):
        sim = sbs.GPUDrainageSimulator(None, 500e-9, W, H)
        set_blocking(sbs, sim, k)
        sim.set_thickness_array(h)
        sim.set_concentration_array(c)
        sim.set_marangoni_enabled(bool(marangoni))
        sim.run(23)
        sim.run(18)
        results.append((sim.thickness_array(), sim.concentration_array()))
    for hk, ck in results[1:]:
        np.testing.assert_array_equal(hk, results[0][0])
        np.testing.assert_array_equal(ck, results[0][1])
    if W * H <= 512 * 200:
        p = orc.wgsl_params(grid_width=W, grid_height=H, marangoni_enabled=marangoni)
        ho, co = orc.wgsl_run(p, h, c, 41, "kernel")
        np.testing.assert_array_equal(results[0][0], ho)
        np.testing.assert_array_equal(results[0][1], co)


def test_time_blocking_keeps_previous_buffer_one_pass_behind(sbs, orc):
    from soap_bubble_simulation_gb300 import synthetic

    h = synthetic.smooth_modes(64, 128).astype(np.float32)
    sim = sbs.GPUDrainageSimulator(None, 500e-9, 128, 64)
    out = ctypes.c_int()
    sbs._native.call("sbs_gpu_drainage_time_blocking", sim.handle, ctypes.byref(out))
    assert out.value == 4
    sim.set_thickness_array(h)
    sim.run(9)  # two 4-step launches and one single step
    prev = orc.wgsl_run(orc.wgsl_params(), h, np.full_like(h, 0.5), 8, "kernel")[0]
    stale = sim.current_buffer()
    v = sbs.film_volume_device(stale.ptr, 64, 128, stale.pitch, 0.025)
    assert v == pytest.approx(orc.film_volume(prev, 0.025), rel=1e-12)


def test_time_blocking_needs_width_multiple_of_4(sbs):
    sim = sbs.GPUDrainageSimulator(None, 500e-9, 130, 20)
    with pytest.raises(sbs.SbsError, match="multiple of 4"):
        set_blocking(sbs, sim, 4)
    set_blocking(sbs, sim, 1)
    sim.run(5)
