"""Parity at the sizes that are timed, against the oracle.

* Config 1 (one bubble at resolution 2048: 2048 x 4096 cells, the benchmark's field), WGSL
  semantics, through the same temporally blocked launches the benchmark runs (4 steps per
  launch, chunks ending at volume checks and at the 256-step graph limit): every cell equal to
  the oracle's kernel-order restatement after 560 steps, the fused FP64 volumes within 1e-12;
  then against drainage.wgsl's own operation order per pass and after 1000 passes.
* Config 1 in CPU semantics (DrainageSimulator, compensated f32x2, TFE on, the first front
  spawning at step 500): every cell equal to the kernel-order oracle after 570 steps; then
  against the f64 restatement of drainage.rs per step and after 1000 steps.
* Config 2 (4,096 bubbles of resolution 32-512, one persistent launch): every bubble equal to
  the single-bubble path after 20 steps, and every resolution-512 bubble plus every 64th bubble
  equal to the oracle.

Against the reference operation order the unmasked error is reported, not bounded: at
resolution 2048 with dt = 1 ms the explicit scheme is unstable in phi on the first ~24 rings at
each pole, those rows blow up and collapse in any run, and two runs that differ in the last bit
diverge there. The bars (1e-5 per step, 1e-4 after 1000 steps) are asserted on the rows the
instability has not reached (parity.stable_rows, with a margin) and on sin(theta) >= 0.2; the
per-step bar also on the rows where one explicit step is stable (parity.cfl_rows): on the others
a single step multiplies the f32 rounding of the Laplacian by the diffusion number (~290 on
ring 1), and the unmasked per-step error of any f32 operation order is ~1e-5 there.
Set SBS_PARITY_LOG to a file path to have the measured errors appended to it as JSON lines.
"""
import json
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

RES = 2048


def log(name, **kw):
    path = os.environ.get("SBS_PARITY_LOG")
    if path:
        with open(path, "a") as f:
            f.write(json.dumps({"test": name, **kw}) + "\n")


def masked(parity, got, ref, initial, **cfl):
    return parity.report(got, ref, initial, cfl)


@pytest.fixture(scope="module")
def c1():
    from soap_bubble_simulation_gb300 import synthetic

    return synthetic.bubble_c1(RES)


def test_c1_wgsl_blocked_bit_exact_and_reference_order(sbs, orc, c1):
    import ctypes

    from soap_bubble_simulation_gb300 import parity

    h, c = c1
    nt, np_ = h.shape
    sim = sbs.GPUDrainageSimulator(None, 550e-9, np_, nt)
    kb = ctypes.c_int()
    sbs._native.call("sbs_gpu_drainage_time_blocking", sim.handle, ctypes.byref(kb))
    assert kb.value == 4
    sim.set_thickness_array(h)
    sim.set_concentration_array(c)
    vols = sim.run_checked(0.0, 300, 100)  # three chunks, each ending in a fused volume check
    sim.run(260)  # a 256-step graph chunk and a 4-step one
    p = orc.wgsl_params(grid_width=np_, grid_height=nt)
    cur = (h, c)
    want_vols = []
    for _ in range(3):
        cur = orc.wgsl_run(p, cur[0], cur[1], 100, "kernel")
        want_vols.append(orc.film_volume(cur[0], 0.025))
    cur = orc.wgsl_run(p, cur[0], cur[1], 260, "kernel")
    got_h, got_c = sim.thickness_array(), sim.concentration_array()
    nbad = int(np.count_nonzero(got_h != cur[0]) + np.count_nonzero(got_c != cur[1]))
    log("c1_wgsl_kernel_order", steps=560, cells_differing=nbad)
    np.testing.assert_array_equal(got_h, cur[0])
    np.testing.assert_array_equal(got_c, cur[1])
    for k in range(3):
        assert vols[k] == pytest.approx(want_vols[k], rel=1e-12)

    # drainage.wgsl's own operation order: one pass from the 560-step state and from the
    # initial field, then 1000 passes from the initial field
    one_gpu = sbs.GPUDrainageSimulator(None, 550e-9, np_, nt)
    per_pass = []
    for src_h, src_c in ((h, c), (got_h, got_c)):
        one_gpu.set_thickness_array(src_h)
        one_gpu.set_concentration_array(src_c)
        one_gpu.run(1)
        w1 = orc.wgsl_run(p, src_h, src_c, 1, "wgsl")
        per_pass.append(masked(parity, one_gpu.thickness_array(), w1[0], h, sin_floor=1e-4))
    sim.run(440)
    wN = orc.wgsl_run(p, h, c, 1000, "wgsl")
    after = masked(parity, sim.thickness_array(), wN[0], h, sin_floor=1e-4)
    cdiff = np.abs(sim.concentration_array().astype(np.float64) - wN[1])
    conc = {"abs": float(cdiff.max()), "abs_sin_ge_0.2": float(cdiff[parity.sin_rows(nt)].max())}
    log("c1_wgsl_reference_order", per_pass=per_pass, after_1000=after, concentration_1000=conc)
    for r in per_pass:
        assert r["rel_linf_cfl_rows"] <= 1e-5, r
        assert r["rel_linf_sin_ge_0.2"] <= 1e-5, r
    assert conc["abs_sin_ge_0.2"] <= 1e-4, conc
    assert after["rel_linf_stable_rows_margin8"] <= 1e-4, after
    assert after["rel_linf_sin_ge_0.2"] <= 1e-4, after
    # the instability is confined to the polar caps
    assert after["stable_rows"] >= nt - 128, after


def test_c1_cpu_semantics_bit_exact_and_f64_reference(sbs, orc, c1):
    from soap_bubble_simulation_gb300 import parity

    h32, _ = c1
    h = h32.astype(np.float64)
    cfg = sbs.SimulationConfig()
    cfg.resolution = RES
    sim = sbs.DrainageSimulator(cfg)
    a = np.ascontiguousarray(h)
    sbs._native.call("sbs_drainage_set_thickness_f64", sim.handle, sbs._native.dptr(a), a.size)
    vols = sim.run_checked(0.001, 300, 100)
    sim.step_n(0.001, 260)
    for _ in range(10):
        sim.step(0.001)
    ref = orc.CpuSim(resolution=RES, precision="f32x2", threads=0)
    ref.set_field(h)
    want_vols = []
    for _ in range(3):
        ref.step_n(0.001, 100)
        want_vols.append(orc.film_volume(ref.field(), cfg.bubble_radius()))
    ref.step_n(0.001, 270)

    def field():
        out = np.empty(h.size)
        sbs._native.call("sbs_drainage_get_thickness_field_f64", sim.handle, sbs._native.dptr(out), out.size)
        return out.reshape(h.shape)

    got, want = field(), ref.field()
    nbad = int(np.count_nonzero(got != want))
    log("c1_cpu_kernel_order", steps=570, cells_differing=nbad, fronts=int(ref.active_tfe_count()))
    assert ref.active_tfe_count() >= 1
    assert sim.active_tfe_count() == ref.active_tfe_count()
    assert sim.current_time() == ref.current_time()
    np.testing.assert_array_equal(got, want)
    for k in range(3):
        assert vols[k] == pytest.approx(want_vols[k], rel=1e-12)

    # the f64 restatement of drainage.rs: one step from the initial field, then 1000 steps
    one = orc.CpuSim(resolution=RES, precision="f64", threads=0)
    one.set_field(h)
    one.step(0.001)
    sim1 = sbs.DrainageSimulator(cfg)
    sbs._native.call("sbs_drainage_set_thickness_f64", sim1.handle, sbs._native.dptr(a), a.size)
    sim1.step(0.001)
    out = np.empty(h.size)
    sbs._native.call("sbs_drainage_get_thickness_field_f64", sim1.handle, sbs._native.dptr(out), out.size)
    per_step = masked(parity, out.reshape(h.shape), one.field(), h)
    sim.step_n(0.001, 430)
    f64 = orc.CpuSim(resolution=RES, precision="f64", threads=0)
    f64.set_field(h)
    f64.step_n(0.001, 1000)
    after = masked(parity, field(), f64.field(), h)
    log("c1_cpu_f64_reference", per_step=per_step, after_1000=after)
    assert per_step["rel_linf_cfl_rows"] <= 1e-5, per_step
    assert per_step["rel_linf_sin_ge_0.2"] <= 1e-5, per_step
    assert after["rel_linf_stable_rows_margin8"] <= 1e-4, after
    assert after["rel_linf_sin_ge_0.2"] <= 1e-4, after
    assert after["stable_rows"] >= RES - 128, after


def test_c2_full_batch_against_single_bubble_path_and_oracle(sbs, orc):
    from soap_bubble_simulation_gb300 import synthetic

    res, rad = synthetic.foam_bubbles()
    hs = synthetic.foam_fields(res)
    foam = sbs.FoamDrainage(res, rad)
    for b in range(len(res)):
        foam.set_thickness(b, hs[b])
    k, rb = foam.autotune(8)
    steps = 20
    foam.run(steps)
    singles = {}
    checked_oracle = 0
    mismatched = []
    for b in range(len(res)):
        r = int(res[b])
        sim = singles.get(r)
        if sim is None:
            sim = singles[r] = sbs.GPUDrainageSimulator(None, 500e-9, 2 * r, r)
        sim.set_bubble_radius(float(rad[b]))
        sim.set_thickness_array(hs[b])
        sim.set_concentration_array(np.full((r, 2 * r), 0.5, np.float32))
        sim.run(steps)
        fh = foam.thickness(b)
        if not (np.array_equal(fh, sim.thickness_array())
                and np.array_equal(foam.concentration(b), sim.concentration_array())):
            mismatched.append(b)
        if r == 512 or b % 64 == 0:
            p = orc.wgsl_params(grid_width=2 * r, grid_height=r, bubble_radius=float(rad[b]))
            oh, oc = orc.wgsl_run(p, hs[b], np.full((r, 2 * r), 0.5, np.float32), steps, "kernel")
            if not (np.array_equal(fh, oh) and np.array_equal(foam.concentration(b), oc)):
                mismatched.append(b)
            checked_oracle += 1
    n512 = int(np.count_nonzero(res == 512))
    log("c2_full_batch", bubbles=int(len(res)), steps=steps, tiles=[k, rb], res512=n512,
        oracle_checked=checked_oracle, mismatched=len(mismatched))
    assert n512 >= 1
    assert not mismatched, f"bubbles differing: {mismatched[:10]}"
