"""Benchmark of the film-drainage path on GB300 (one JSON line on stdout).

Workload (the plain method at scale): one bubble at resolution 2048 (2048 theta x 4096 phi =
8.4 M cells), f32 thickness h = 550 nm + 16 seeded smooth modes clamped to [100, 1000] nm,
surfactant 0.5 +- 0.1, reference fluid defaults, dt 1 ms. A bench step is one full run of
10,000 drainage steps of the GPUDrainageSimulator semantics (h and surfactant co-evolve,
drainage.wgsl) with the FP64 film-volume check fused into every 100th step. Inputs are
synthetic (seeded); the field keeps evolving from step to step. L2 (129 MB) is flushed with a
512 MB write before every bench step.

value: cell-steps/s over the K timed bench steps, device-resident, CUDA events on the
handle's stream. e2e: the same through the C ABI with host buffers: each step uploads h and
surfactant from pinned host memory, runs, and reads both fields and the volumes back.
roofline: the dominant kernel, the temporally blocked step (wtb_wgsl_kernel, 4 steps per
launch), at 16 algorithmic bytes per cell-step (read h, Gamma; write h, Gamma) times the steps
of a launch, against the measured copy bandwidth; `traffic` is its ncu DRAM bytes per launch.
cpu_baseline: the oracle's restatement of drainage.wgsl (the same semantics: f32 h and
surfactant, drainage.wgsl's own operation order) on all host cores, on a bounded sample of the
same field (about --cpu-seconds of work); cpu_baseline_single_thread: the same on one core.
parity: the GPU field after the baseline sample's number of passes against the sample's
result (relative L-inf unmasked and on the CFL-stable rows, the rows the polar instability has
not reached and sin(theta) >= 0.2), and 100 passes bit for bit against the oracle's restatement
of the kernels' operation order.
cpu_semantics: the reference's own solver, DrainageSimulator::step (pole means, fronts), at the
same size: compensated f32x2 (16 B per cell-step; also given at 8 B, h only) and plain f32, with
the f64 restatement of drainage.rs:298-503 on all host cores beside it.
res4096: the WGSL step at 4096 x 8192 cells (537 MB, four times L2).
surrogate: the learned 64-step operator (include/sbs_nn.h) trained here on 512 plain-solver
trajectories at 256 x 512, then a 10,000-step rollout of the same 2048 x 4096 field with a plain
check every 8 intervals; effective cell-steps/s and the masked relative L-inf error of the final
thickness against the plain run (rows with sin(theta) >= 0.2; nearer the poles the explicit
scheme is unstable at this resolution). `surrogate` is the network with GELU activations (the
default), `surrogate_hswish` the same network, data and schedule with hard-swish.
foam / spectral: the batched-foam and spectral-contraction workloads, device-resident.
c0: the small configuration's latency-bound calls (1000 steps at resolution 128 in both
semantics, the colour LUTs, colours at 10,242 icosphere vertices), host in and host out.
shading: one 3840 x 2160 headless frame of the bubble fragment shader, pixels/s.
caustics: the caustic pass over the drained 2048 x 4096 field, on the simulator's device field.
branched_flow: one step of the branched-flow ray tracer at the reference's defaults.
foam_dynamics: FoamSimulator::step over a 1,048,576-bubble FCC foam (and 4,096 bubbles beside the
oracle's all-pairs loops on one host core), bubble-steps/s.

--impl reference: times the drainage.wgsl restatement alone on all host cores (the reference is
Rust and WGSL; neither can run here), same metric, config and semantics.

The line ends with `summary`: the headline figures of every section, rounded.
"""
from __future__ import annotations

import argparse
import ctypes
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

RES = 2048
STEPS_PER_RUN = 10_000
CHECK_EVERY = 100
BYTES_PER_CELL_STEP = 16  # read h + Gamma, write h + Gamma (f32)
METRIC = "drainage cell-steps/s, plain vs surrogate at <=1e-3 rel h error; % HBM roofline"


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=3)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="ours", choices=["ours", "reference"])
    p.add_argument("--cpu-seconds", type=float, default=20.0, help="target CPU baseline sample length")
    p.add_argument("--skip-aux", action="store_true",
                   help="plain path only (no surrogate / foam / spectral / CPU baseline), e.g. for an ncu launch list")
    return p.parse_args()


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def max_over_ranks(*vals):
    """Each value's maximum over the ranks (one all-reduce over the process group; the values
    themselves for a single process): the slowest replica's times set the whole-job rate."""
    import torch

    t = torch.tensor(vals, dtype=torch.float64)
    dist = torch.distributed
    if dist.is_available() and dist.is_initialized() and dist.get_world_size() > 1:
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return [float(x) for x in t]


def hbm_peak():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def ncu_traffic():
    """Per-launch DRAM bytes of the step kernel from the committed ncu summary (or None)."""
    path = os.path.join(ROOT, "profiles", "drain_wtb_wgsl_c1.md")
    try:
        for line in open(path):
            if line.startswith("traffic_bytes_per_launch:"):
                return int(float(line.split(":", 1)[1]))
    except OSError:
        pass
    return None


class ClockSampler:
    """nvidia-smi clock/throttle samples while the timed region runs."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.rows = []
        self.proc = None
        self.gpu = gpu_index

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([x.strip() for x in line.split(",")])

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm = [float(r[1]) for r in self.rows if len(r) > 2 and r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in self.rows if len(r) > 2 and r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = set()
        for r in self.rows:
            for i, n in enumerate(names):
                if len(r) > 5 + i and r[5 + i].lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(self.rows)}


def workload_config(world: int) -> dict:
    """The workload both arms report (the same dict, so the driver can compare them)."""
    return {"workload": "bubble resolution 2048 (2048 theta x 4096 phi = 8.4M cells), h 550 nm + 16 seeded modes, "
                        "surfactant 0.5+-0.1, fluid defaults, dt 1e-3 s, 10,000 steps of GPUDrainageSimulator "
                        "semantics (drainage.wgsl: f32 h and surfactant) per bench step, FP64 volume check every 100 "
                        "steps",
            "cells": RES * 2 * RES, "drainage_steps_per_bench_step": STEPS_PER_RUN, "check_every": CHECK_EVERY,
            "l2": "512 MB write before every bench step (working set 128 MB)", "replicas": world}


def _oracle():
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as orc

    return orc


def cpu_baseline(h: np.ndarray, c: np.ndarray, target_s: float, threads: int):
    """The oracle's restatement of drainage.wgsl (drainage.wgsl:72-202, its own f32 operation order,
    h and surfactant) on `threads` host cores over a bounded sample of the workload. Returns the
    baseline record and the sample's final fields (for the parity check)."""
    orc = _oracle()
    nt, np_ = h.shape
    p = orc.wgsl_params(grid_width=np_, grid_height=nt)
    t0 = time.perf_counter()
    orc.wgsl_run(p, h, c, 1, "wgsl", threads)
    one = time.perf_counter() - t0
    n = int(max(2, min(20000, target_s / max(one, 1e-6))))
    t0 = time.perf_counter()
    hn, cn = orc.wgsl_run(p, h, c, n, "wgsl", threads)
    dt = time.perf_counter() - t0
    rec = {"value": h.size * n / dt, "unit": "cell-steps/s", "cores": threads, "kind": "port",
           "sample": f"{n} passes of drainage_step (drainage.wgsl:72-202, f32 h and surfactant, its own operation "
                     f"order) on the 2048 x 4096 field, {dt:.1f} s"}
    return rec, (n, hn, cn)


def cpu_baseline_f64(h: np.ndarray, target_s: float, threads: int):
    """The oracle's f64 restatement of DrainageSimulator::step (drainage.rs:298-503) over a bounded sample."""
    orc = _oracle()
    sim = orc.CpuSim(resolution=h.shape[0], precision="f64", threads=threads)
    sim.set_field(h.astype(np.float64))
    t0 = time.perf_counter()
    sim.step(0.001)
    one = time.perf_counter() - t0
    n = int(max(2, min(20000, target_s / max(one, 1e-6))))
    t0 = time.perf_counter()
    sim.step_n(0.001, n)
    dt = time.perf_counter() - t0
    return {"value": h.size * n / dt, "unit": "cell-steps/s", "cores": threads, "kind": "port",
            "sample": f"{n} steps of DrainageSimulator::step (f64, drainage.rs:298-503) on the 2048 x 4096 field, "
                      f"{dt:.1f} s"}


def parity_section(sbs, sample, h0, c0):
    """The GPU path against the CPU sample's fields (same input, same number of passes), and 100
    passes bit for bit against the oracle's restatement of the kernels' own operation order."""
    from soap_bubble_simulation_gb300 import parity

    orc = _oracle()
    n, hn, _ = sample
    nt, np_ = h0.shape
    sim = sbs.GPUDrainageSimulator(None, 550e-9, np_, nt)
    sim.set_thickness_array(h0)
    sim.set_concentration_array(c0)
    sim.run(100)
    hk, ck = orc.wgsl_run(orc.wgsl_params(grid_width=np_, grid_height=nt), h0, c0, 100, "kernel")
    differing = int(np.count_nonzero(sim.thickness_array() != hk) + np.count_nonzero(sim.concentration_array() != ck))
    sim.run(n - 100)
    r = parity.report(sim.thickness_array(), hn, h0, {"sin_floor": 1e-4})
    sim.close()
    return {"steps": n, "reference": "drainage.wgsl operation order (f32)", **r,
            "kernel_order_cells_differing_after_100": differing}


def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return
    from soap_bubble_simulation_gb300 import synthetic

    h, c = synthetic.bubble_c1(RES)
    threads = os.cpu_count() or 1
    for _ in range(args.warmup):
        cpu_baseline(h, c, 0.3, threads)
    vals = [cpu_baseline(h, c, args.cpu_seconds / max(args.steps, 1), threads)[0] for _ in range(args.steps)]
    v = statistics.median(x["value"] for x in vals)
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": "cell-steps/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": h.size * STEPS_PER_RUN / v * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": workload_config(world),
            "cpu_baseline": {**vals[-1], "value": v},
            "e2e": {"value": v, "unit": "cell-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def launches_per_run(k: int) -> int:
    """Kernel launches of one run of STEPS_PER_RUN steps with a volume check every CHECK_EVERY (the
    library's chunking: chunks end at each check; within a chunk k-step launches, then single
    steps for the remainder, the run's very last step single)."""
    total, done = 0, 0
    while done < STEPS_PER_RUN:
        g = min(256, STEPS_PER_RUN - done, CHECK_EVERY - done % CHECK_EVERY)
        tail = 1 if done + g == STEPS_PER_RUN else 0
        body = g - tail
        total += (body // k + body % k + tail) if k > 1 else g
        done += g
    return total


def surrogate_section(sbs, synthetic, h0, c0, torch, activations=("gelu", "hswish")):
    """C4: train on 480 plain trajectories at 256 x 512 (config-1 fields, mirrored and step windows of
    2048-resolution fields), evaluate on 24 held-out continuous and 8 held-out step trajectories, then
    the checked 10,000-step rollout, once per activation (GELU, the network's default, and hard-swish)
    from the same initial weights and data."""
    nt, np_ = h0.shape
    cells = h0.size
    s = sbs.DrainageSurrogate(seed=7)
    theta0 = s.params
    t0 = time.perf_counter()
    ntrain, nheld, nstep = 480, 24, 8
    ntraj = ntrain + nheld + nstep
    # training trajectories of every kind, then held-out continuous films (config-1 fields and
    # mirrored windows) and held-out step windows, each a contiguous block for evaluate()
    sets = ((ntrain, 21, synthetic.SURROGATE_KINDS), (nheld, 22, ("c1", "mirror")), (nstep, 23, ("step",)))
    for count, seed, kinds in sets:
        for h, c, visc, rad in synthetic.surrogate_trajectories(count, seed=seed, kinds=kinds):
            s.add_trajectory(h, c, sbs.field_params(256, 512, viscosity=visc, bubble_radius=rad), pairs=4)
    data_s = time.perf_counter() - t0
    p = sbs.field_params(nt, np_, bubble_radius=0.025)

    def fresh():
        sim = sbs.GPUDrainageSimulator(None, 550e-9, np_, nt)
        sim.update_params(p)
        sim.set_thickness_array(h0)
        sim.set_concentration_array(c0)
        return sim

    # plain reference run (same stream semantics as the rollout's plain intervals, no volume checks)
    # every timed run is first run once untimed on the same handle (graph captures, scratch, first
    # kernel loads), then restarted from the same fields
    ref = fresh()
    ref.run(STEPS_PER_RUN)
    ref.set_thickness_array(h0)
    ref.set_concentration_array(c0)
    torch.cuda.synchronize()
    ta = time.perf_counter()
    ref.run(STEPS_PER_RUN)
    torch.cuda.synchronize()
    plain_s = time.perf_counter() - ta
    h_ref = ref.thickness_array()
    ref.close()
    err_id = sbs.masked_error(h0, h_ref)
    peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json"))) if os.path.exists(
        os.path.join(ROOT, "MEASURED_PEAKS.json")) else {}
    tf_peak = float(peaks.get("bf16_tflops", 1900.0))
    flop_cell = 2 * 9 * (16 * 32 + 32 * 32 * 2 + 32 * 1)  # useful multiply-adds x 2 per cell and interval
    # a training iteration per cell: the forward pass, every layer's weight gradient (as many
    # multiply-adds as the forward pass) and the input gradients of layers 2-4
    train_flop_cell = 2 * flop_cell + 2 * 9 * (32 * 32 * 2 + 32 * 1)
    plain_rate = cells * STEPS_PER_RUN / plain_s
    iters = 3000
    results = {}
    for act in activations:
        s.activation = act
        s.params = theta0  # same start for every activation (also resets the optimiser state)
        t1 = time.perf_counter()
        losses = s.train(ntrain, iters, batch=8, lr=2e-3, seed=5)
        torch.cuda.synchronize()
        t2 = time.perf_counter()
        ev = s.evaluate(ntrain, nheld, mode="fused")
        ev_step = s.evaluate(ntrain + nheld, nstep, mode="fused")
        # fused forward pass alone (one 64-pass interval)
        sim = fresh()
        for _ in range(3):
            s.advance(sim, mode="fused")
        reps = 20
        torch.cuda.synchronize()
        ta = time.perf_counter()
        for _ in range(reps):
            s.advance(sim, mode="fused")
        torch.cuda.synchronize()
        fused_ms = (time.perf_counter() - ta) / reps * 1e3
        sim.close()
        # the checked rollout: 156 intervals (9,984 passes) + 16 plain passes = 10,000 steps
        sim = fresh()
        s.rollout(sim, STEPS_PER_RUN // 64 * 64, check_every=8, tol=1e-3, mode="fused")
        sim.run(STEPS_PER_RUN % 64)
        sim.set_thickness_array(h0)
        sim.set_concentration_array(c0)
        torch.cuda.synchronize()
        ta = time.perf_counter()
        st = s.rollout(sim, STEPS_PER_RUN // 64 * 64, check_every=8, tol=1e-3, mode="fused")
        sim.run(STEPS_PER_RUN % 64)
        torch.cuda.synchronize()
        roll_s = time.perf_counter() - ta
        err = sbs.masked_error(sim.thickness_array(), h_ref)
        sim.close()
        tflops = flop_cell * cells / (fused_ms * 1e-3) / 1e12
        rate = cells * STEPS_PER_RUN / roll_s
        results[act] = {
            "activation": act, "value": rate, "unit": "cell-steps/s", "speedup_vs_plain": rate / plain_rate,
            "plain_value": plain_rate, "masked_rel_linf_vs_plain": err, "identity_rel_linf_vs_plain": err_id,
            "tol": 1e-3, "stats": st, "fused_ms_per_interval": fused_ms,
            "fused_interval_cell_steps_per_s": cells * 64 / (fused_ms * 1e-3),
            "tensor": {"bound": "tensor", "achieved": tflops, "peak": tf_peak, "unit": "TFLOP/s",
                       "frac": tflops / tf_peak, "flop_per_cell": flop_cell, "peak_kind": "measured bf16 burst"},
            "train": {"trajectories": ntrain, "kinds": list(synthetic.SURROGATE_KINDS), "grid": "256 x 512",
                      "pairs_per_trajectory": 4, "iters": iters,
                      "ms_per_iter": (t2 - t1) * 1e3 / iters,
                      "tflops": train_flop_cell * 8 * 256 * 512 * iters / (t2 - t1) / 1e12,
                      "flop_per_cell_iter": train_flop_cell,
                      "batch": 8, "data_s": data_s, "train_s": t2 - t1, "loss_first": float(losses[:10].mean()),
                      "loss_last": float(losses[-50:].mean())},
            "heldout_256": {**ev, "trajectories": nheld, "kinds": ["c1", "mirror"]},
            "heldout_256_step": {**ev_step, "trajectories": nstep, "kinds": ["step"]}}
    s.close()
    return results


def foam_section(sbs, synthetic, torch):
    res, rad = synthetic.foam_bubbles()
    foam = sbs.FoamDrainage(res, rad)
    hs = synthetic.foam_fields(res)
    for b in range(len(res)):
        foam.set_thickness(b, hs[b])
    k, rb = foam.autotune(8)
    foam.run(100)
    st = torch.cuda.ExternalStream(foam.stream())
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record(st)
    foam.run(1000)
    b.record(st)
    torch.cuda.synchronize()
    ms = a.elapsed_time(b)
    cells = foam.total_cells()
    foam.close()
    return {"value": cells * 1000 / (ms * 1e-3), "unit": "cell-steps/s", "bubbles": int(len(res)), "cells": int(cells),
            "steps": 1000, "ms": ms, "tiles": {"steps_per_phase": k, "strip_rows": rb},
            "algorithmic_gbs": cells * 1000 * 16 / (ms * 1e-3) / 1e9}


def c0_section(sbs, synthetic, torch):
    """C0, latency-bound: 1000 steps at resolution 128 (128 x 256 cells) in both semantics, the
    256 x 64 colour LUT over 0-1000 nm, the RGBA8 LUT and colours at the 10,242 subdivision-5
    icosphere vertices, each timed through the public call (host in, host out)."""

    def best(fn, reps=5):
        fn()
        ts = []
        for _ in range(reps):
            ta = time.perf_counter()
            fn()
            ts.append(time.perf_counter() - ta)
        return min(ts)

    cfg = sbs.SimulationConfig()
    cfg.resolution = 128
    h = synthetic.bubble_c0(128, seed=0)
    cpu = sbs.DrainageSimulator(cfg)

    def run_cpu():
        cpu.set_thickness_array(h)
        cpu.step_n(cfg.dt, 1000)

    t_cpu = best(run_cpu)
    gpu = sbs.GPUDrainageSimulator(None, 500e-9, 256, 128)

    def run_gpu():
        gpu.set_thickness_array(h.astype(np.float32))
        gpu.run(1000)

    t_gpu = best(run_gpu)
    calc = sbs.InterferenceCalculator(1.33)
    lut = calc.color_lookup_2d_array(0.0, 1000.0, 256, 64)
    t_lut = best(lambda: calc.color_lookup_2d_array(0.0, 1000.0, 256, 64))
    t_rgba = best(lambda: sbs.generate_interference_lut(1.33, 1.0))
    xyz = synthetic.icosphere(5)
    t_vert = best(lambda: cpu.vertex_colors(xyz, lut, 0.0, 1000.0))
    cells = 128 * 256
    cpu.close()
    gpu.close()
    return {"drainage_cpu_semantics": {"ms_per_1000_steps": t_cpu * 1e3, "cell_steps_per_s": cells * 1000 / t_cpu},
            "drainage_wgsl_semantics": {"ms_per_1000_steps": t_gpu * 1e3, "cell_steps_per_s": cells * 1000 / t_gpu},
            "lut_256x64_f64": {"ms": t_lut * 1e3, "points_per_s": 256 * 64 / t_lut},
            "lut_rgba8_64x256": {"ms": t_rgba * 1e3, "texels_per_s": 256 * 64 / t_rgba},
            "vertex_colors": {"vertices": int(len(xyz)), "ms": t_vert * 1e3, "points_per_s": len(xyz) / t_vert}}


def shade_section(sbs, torch):
    """Headless film shading: one 3840 x 2160 frame of the bubble fragment shader (RGBA8 sRGB out),
    camera at 6 cm so that the bubble covers most of the frame; device-resident (CUDA events) and
    through the host call (frame copied back)."""
    from soap_bubble_simulation_gb300 import shading as sh

    N = sbs._native
    w, h = 3840, 2160
    u = sh.BubbleUniform.default()
    u.set_time(2.0)
    cam = sh.Camera(aspect=w / h, distance=0.06)
    vp, pos = cam.view_proj(), cam.position().astype(np.float32)
    lut = torch.from_numpy(sh.default_lut(1.33).copy()).cuda()
    out8 = torch.empty((h, w, 4), dtype=torch.uint8, device="cuda")
    st = torch.cuda.current_stream()

    def run():
        N.call("sbs_shade_frame", ctypes.cast(ctypes.byref(u), ctypes.c_void_p), N.ptr(vp), N.ptr(pos),
               float(sh.HEADLESS_RADIUS), ctypes.c_void_p(lut.data_ptr()), None, w, h,
               ctypes.c_void_p(out8.data_ptr()), None, N.MEM_DEVICE, ctypes.c_void_p(st.cuda_stream))

    for _ in range(3):
        run()
    reps = 20
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record(st)
    for _ in range(reps):
        run()
    b.record(st)
    torch.cuda.synchronize()
    ms = a.elapsed_time(b) / reps
    frame = out8.cpu().numpy()
    bg = np.array([round(255 * (1.055 * x ** (1 / 2.4) - 0.055)) for x in (0.1, 0.1, 0.15)])
    cover = float(np.any(frame[..., :3] != bg, axis=-1).mean())
    sh.render_frame(u, cam, w, h)
    ta = time.perf_counter()
    for _ in range(5):
        sh.render_frame(u, cam, w, h)
    e2e_ms = (time.perf_counter() - ta) / 5 * 1e3
    return {"value": w * h / (ms * 1e-3), "unit": "pixels/s", "ms_per_frame": ms, "frame": f"{w} x {h}",
            "bubble_coverage": cover, "bytes_out_per_pixel": 4,
            "e2e": {"value": w * h / (e2e_ms * 1e-3), "unit": "pixels/s", "ms_per_frame": e2e_ms,
                    "d2h_bytes_per_frame": 4 * w * h}}


def caustics_section(sbs, synthetic, torch, h0, c0):
    """The caustic pass over the 2048 x 4096 field after a drainage run, on the simulator's own
    device field (no copy): 8 algorithmic bytes per cell (read h, write the map); then runs of 10
    and 100 passes with the map of the buffer the renderer binds, separate pass against the map
    written by the run's final blocked launch."""
    from soap_bubble_simulation_gb300.caustics import CausticParams

    N = sbs._native
    nt, np_ = h0.shape
    sim = sbs.GPUDrainageSimulator(None, 550e-9, np_, nt)
    sim.set_thickness_array(h0)
    sim.set_concentration_array(c0)
    sim.run(100)
    p = CausticParams.default(np_, nt)
    out = torch.empty((nt, np_), device="cuda")
    st = torch.cuda.ExternalStream(sim.stream())

    def run():
        N.call("sbs_gpu_drainage_caustics", sim.handle, ctypes.cast(ctypes.byref(p), ctypes.c_void_p), 0,
               ctypes.c_void_p(out.data_ptr()), N.MEM_DEVICE)

    for _ in range(3):
        run()
    reps = 50
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record(st)
    for _ in range(reps):
        run()
    b.record(st)
    torch.cuda.synchronize()
    ms = a.elapsed_time(b) / reps

    # a run of drainage passes and the map of the buffer the renderer binds: run() then the separate
    # pass, against run_caustics (the map written by the run's final blocked launch)
    pp = ctypes.cast(ctypes.byref(p), ctypes.c_void_p)
    outp = ctypes.c_void_p(out.data_ptr())

    def frame(fused, passes):
        if fused:
            N.call("sbs_gpu_drainage_run_caustics", sim.handle, passes, pp, outp, N.MEM_DEVICE)
        else:
            N.call("sbs_gpu_drainage_run", sim.handle, passes)
            N.call("sbs_gpu_drainage_caustics", sim.handle, pp, 1, outp, N.MEM_DEVICE)

    fused_runs = {}
    for passes in (10, 100):
        res = {}
        for fused in (False, True):
            for _ in range(3):
                frame(fused, passes)
            n = 20
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            torch.cuda.synchronize()
            e0.record(st)
            for _ in range(n):
                frame(fused, passes)
            e1.record(st)
            torch.cuda.synchronize()
            res["fused_us" if fused else "separate_us"] = e0.elapsed_time(e1) / n * 1e3
        res["saved_us"] = res["separate_us"] - res["fused_us"]
        fused_runs[f"passes_{passes}"] = res
    sim.close()
    peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json"))) if os.path.exists(
        os.path.join(ROOT, "MEASURED_PEAKS.json")) else {}
    hbm_peak = float(peaks.get("hbm_gbs", 6800.0))
    gbs = 8.0 * h0.size / (ms * 1e-3) / 1e9
    return {"value": h0.size / (ms * 1e-3), "unit": "cells/s", "us_per_map": ms * 1e3, "grid": f"{nt} x {np_}",
            "hbm": {"achieved": gbs, "peak": hbm_peak, "unit": "GB/s", "frac": gbs / hbm_peak,
                    "bytes_per_cell": 8},
            "run_and_map": fused_runs}


def branched_section(sbs, synthetic, torch):
    """Branched flow: one step of the reference's defaults (32,768 rays x 400 kick-drift steps, 800
    scatterers, 512 x 256 texture; patch off so that every step deposits) over a 128 x 64 film,
    device-resident (CUDA events) and through the host call."""
    from soap_bubble_simulation_gb300 import branched as br

    N = sbs._native
    p = br.BranchedFlowParams.default()
    p.patch_enabled = 0
    th = (synthetic.smooth_modes(64, 128, seed=3) * 2e4).astype(np.float32)
    sc = br.generate_scatterers(p, time=1.5)
    dth, dsc = torch.from_numpy(th).cuda(), torch.from_numpy(sc).cuda()
    dtex = torch.zeros((p.tex_height, p.tex_width), dtype=torch.int32, device="cuda")
    st = torch.cuda.current_stream()

    def run():
        N.call("sbs_branched_flow", ctypes.cast(ctypes.byref(p), ctypes.c_void_p), ctypes.c_void_p(dth.data_ptr()),
               128, 64, 128, ctypes.c_void_p(dsc.data_ptr()), ctypes.c_void_p(dtex.data_ptr()), 1, N.MEM_DEVICE,
               ctypes.c_void_p(st.cuda_stream))

    for _ in range(2):
        run()
    reps = 10
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record(st)
    for _ in range(reps):
        run()
    b.record(st)
    torch.cuda.synchronize()
    ms = a.elapsed_time(b) / reps
    tex = np.zeros((p.tex_height, p.tex_width), np.uint32)
    br.branched_flow_step(p, th, sc, tex)
    ta = time.perf_counter()
    for _ in range(3):
        tex = br.branched_flow_step(p, th, sc, tex)
    e2e_ms = (time.perf_counter() - ta) / 3 * 1e3
    steps = p.num_rays * p.ray_steps
    return {"value": steps / (ms * 1e-3), "unit": "ray-steps/s", "ms_per_step": ms, "rays": int(p.num_rays),
            "steps_per_ray": int(p.ray_steps), "scatterers": int(p.num_scatterers),
            "e2e": {"value": steps / (e2e_ms * 1e-3), "unit": "ray-steps/s", "ms_per_step": e2e_ms}}


def foam_dynamics_section(sbs, cpu_seconds: float):
    """Foam cluster dynamics (FoamSimulator::step): a face-centred cubic foam of 1,048,576 bubbles
    (FoamGenerator::generate_fcc's layout, spacing 5 cm, radii 1.5-3 cm, jitter 0.1, seeded),
    dt = 1 ms, 200 steps timed in one call (the neighbour list is rebuilt about every 70 steps at
    this dt, so the rebuilds are included at their rate); e2e adds the per-frame read-back of every bubble's
    position, velocity, radius and thickness. The same at 4,096 bubbles next to the oracle's
    restatement of the reference's all-pairs loops on one host core (the reference is
    single-threaded), timed on a bounded number of steps."""
    from soap_bubble_simulation_gb300 import foam_dynamics as fd

    out = {}
    for n, k in ((1_048_576, 200), (4096, 1000)):
        pos, rad = fd.fcc_foam(n, seed=0)
        sim = fd.FoamSimulator(pos, rad)
        sim.step(1e-3, 3)
        t0 = time.perf_counter()
        sim.step(1e-3, k)
        ms = (time.perf_counter() - t0) / k * 1e3
        reps = 5 if n > 10000 else 50
        t0 = time.perf_counter()
        for _ in range(reps):
            sim.step(1e-3)
            sim.bubbles()
        e2e_ms = (time.perf_counter() - t0) / reps * 1e3
        out[n] = {"bubbles": n, "ms_per_step": ms, "value": n / (ms * 1e-3), "unit": "bubble-steps/s",
                  "connections": sim.connection_count(),
                  "e2e": {"value": n / (e2e_ms * 1e-3), "unit": "bubble-steps/s", "ms_per_step": e2e_ms,
                          "d2h_bytes_per_step": n * 36}}
        sim.close()
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as orc

    pos, rad = fd.fcc_foam(4096, seed=0)
    phys = fd.FoamPhysics.default()
    r = orc.foam_step(phys, 1e-3, 1, pos, rad)
    steps, t0 = 0, time.perf_counter()
    while time.perf_counter() - t0 < cpu_seconds:
        r = orc.foam_step(phys, 1e-3, 1, r["position"], r["radius"], velocity=r["velocity"], ids=r["ids"],
                          next_id=r["next_id"])
        steps += 1
    cpu_ms = (time.perf_counter() - t0) / steps * 1e3
    big, small = out[1_048_576], out[4096]
    return {"value": big["value"], "unit": "bubble-steps/s", "ms_per_step": big["ms_per_step"],
            "bubbles": big["bubbles"], "connections": big["connections"], "e2e": big["e2e"],
            "small": small,
            "cpu_baseline": {"value": 4096 / (cpu_ms * 1e-3), "unit": "bubble-steps/s", "cores": 1, "kind": "port",
                             "sample": f"4,096 bubbles, {steps} steps of the all-pairs loops", "ms_per_step": cpu_ms}}


def spectral_section(sbs, synthetic, torch):
    N = sbs._native
    n = 8_388_608
    t, c, nf = synthetic.spectral_points(n)
    wl = synthetic.WAVELENGTHS_81.astype(np.float32)
    cmf = synthetic.spectral_cmf().astype(np.float32)
    dt, dc, dn = (torch.from_numpy(x).cuda() for x in (t, c, nf))
    peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json"))) if os.path.exists(
        os.path.join(ROOT, "MEASURED_PEAKS.json")) else {}
    hbm_peak = float(peaks.get("hbm_gbs", 6800.0))
    tf_peak = float(peaks.get("bf16_tflops", 1900.0))
    out = {}
    res = {}
    for mode, name in ((N.SPECTRAL_TC_BF16, "tc_bf16"), (N.SPECTRAL_FP32, "fp32")):
        o = torch.empty((n, 3), device="cuda")

        def run():
            N.call("sbs_spectral_rgb", ctypes.c_void_p(dt.data_ptr()), ctypes.c_void_p(dc.data_ptr()),
                   ctypes.c_void_p(dn.data_ptr()), n, N.ptr(wl), wl.size, N.ptr(cmf), mode,
                   ctypes.c_void_p(o.data_ptr()), N.MEM_DEVICE, None)

        run()
        torch.cuda.synchronize()
        reps = 10
        ta = time.perf_counter()
        for _ in range(reps):
            run()
        torch.cuda.synchronize()
        ms = (time.perf_counter() - ta) / reps * 1e3
        # roofline fractions: HBM at 24 B per point (t, cos, n in; RGB out), the contraction's 486
        # useful FLOP per point on the tensor pipe; the bound is the FP32 / SFU work of the 81 Airy
        # terms per point (ncu: FMA pipe ~64 % of active cycles, profiles/spectral_tc_c3.md)
        gbs = 24.0 * n / (ms * 1e-3) / 1e9
        tfl = 2.0 * 81 * 3 * n / (ms * 1e-3) / 1e12
        out[name] = {"value": n / (ms * 1e-3), "unit": "points/s", "ms": ms,
                     "hbm": {"achieved": gbs, "peak": hbm_peak, "unit": "GB/s", "frac": gbs / hbm_peak},
                     "tensor": {"achieved": tfl, "peak": tf_peak, "unit": "TFLOP/s", "frac": tfl / tf_peak,
                                "pipe": "tcgen05 BF16" if name == "tc_bf16" else "none (FP32 FMA contraction)"},
                     "bound": "FP32/SFU: spectrum generation (81 Airy terms per point)"}
        res[name] = o[:262144].cpu().numpy()
    # precision on a 262,144-point subset against the FP64 oracle
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as orc

    m = 262144
    want = orc.spectral_rgb(t[:m], c[:m], nf[:m], wl.astype(np.float64), cmf.astype(np.float64))
    for name in res:
        rel = float(np.max(np.abs(res[name] - want)) / np.max(np.abs(want)))
        de = synthetic.delta_e76(res[name], want, cmf.astype(np.float64).sum(0))
        out[name].update({"rel_linf_vs_fp64": rel, "delta_e76_mean": float(de.mean()), "delta_e76_max": float(de.max())})
    out["points"] = n
    out["wavelengths"] = int(wl.size)
    return out


def profile_traffic(name: str):
    """`traffic_bytes_per_launch:` of a committed ncu summary under profiles/ (or None)."""
    try:
        for line in open(os.path.join(ROOT, "profiles", name)):
            if line.startswith("traffic_bytes_per_launch:"):
                return int(float(line.split(":", 1)[1]))
    except OSError:
        pass
    return None


def cpu_semantics_section(sbs, torch, h0, peak, cpu_seconds):
    """The reference's own solver (DrainageSimulator::step with pole means and fronts) at 2048 x 4096
    on the GPU, compensated f32x2 (the default) and plain f32, timed over 2000 steps after 512
    (fronts active from step 500), with its roofline and the f64 restatement on all host cores."""
    from soap_bubble_simulation_gb300 import _native as N

    cells = h0.size
    out = {}
    for prec, bpc in (("f32x2", 16), ("f32", 8)):
        cfg = sbs.SimulationConfig()
        cfg.resolution = RES
        c = cfg.to_c()
        hh = ctypes.c_void_p()
        N.call("sbs_drainage_create_ex", ctypes.byref(c), N.DRAIN_F32X2 if prec == "f32x2" else N.DRAIN_F32,
               ctypes.byref(hh))
        sim = sbs.DrainageSimulator.__new__(sbs.DrainageSimulator)
        sbs.drainage._Handle.__init__(sim)
        sim._h = hh
        sim._config = cfg
        kb = ctypes.c_int()
        N.call("sbs_drainage_time_blocking", sim.handle, ctypes.byref(kb))
        sim.set_thickness_array(h0)
        sim.step_n(0.001, 512)
        st = torch.cuda.ExternalStream(sim.stream())
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        n = 2000
        torch.cuda.synchronize()
        a.record(st)
        sim.step_n(0.001, n)
        b.record(st)
        torch.cuda.synchronize()
        ms = a.elapsed_time(b)
        sim.close()
        rate = cells * n / (ms * 1e-3)
        gbs = bpc * rate / 1e9
        out[prec] = {"value": rate, "unit": "cell-steps/s", "us_per_step": ms * 1e3 / n, "steps_per_launch": kb.value,
                     "roofline": {"bound": "hbm", "bytes_per_cell_step": bpc, "achieved": gbs, "peak": peak,
                                  "unit": "GB/s", "frac": gbs / peak,
                                  "frac_at_8B_per_cell_step": 8 * rate / 1e9 / peak,
                                  "traffic": profile_traffic("drain_wtbc_cpu_c1.md") if prec == "f32x2" else None,
                                  "kernel": f"wtbc_kernel<{kb.value}, {'compensated' if prec == 'f32x2' else 'f32'}>"}}
    base = cpu_baseline_f64(h0, cpu_seconds, os.cpu_count() or 1)
    out["cpu_baseline"] = base
    out["vs_cpu_baseline"] = out["f32x2"]["value"] / base["value"]
    return out


def res4096_section(sbs, synthetic, torch, peak):
    """The WGSL step at resolution 4096 (4096 x 8192 cells, a 537 MB working set: 4 x the 129 MB
    L2), where the temporally blocked kernel's fields cannot stay in L2 between launches."""
    h, c = synthetic.bubble_c1(4096)
    nt, np_ = h.shape
    sim = sbs.GPUDrainageSimulator(None, 550e-9, np_, nt)
    sim.set_thickness_array(h)
    sim.set_concentration_array(c)
    sim.run(40)
    st = torch.cuda.ExternalStream(sim.stream())
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    n = 400
    torch.cuda.synchronize()
    a.record(st)
    sim.run(n)
    b.record(st)
    torch.cuda.synchronize()
    ms = a.elapsed_time(b)
    sim.close()
    rate = h.size * n / (ms * 1e-3)
    launch_us = ms * 1e3 / n * 4
    dram = 511_542_272  # ncu DRAM bytes per 4-step launch at this size (profiles/drain_wtb_wgsl_c1.md)
    return {"value": rate, "unit": "cell-steps/s", "cells": int(h.size), "steps": n, "launch_us": launch_us,
            "roofline": {"bound": "hbm", "achieved": 16 * rate / 1e9, "peak": peak, "unit": "GB/s",
                         "frac": 16 * rate / 1e9 / peak, "traffic": dram,
                         "dram_frac": dram / (launch_us * 1e-6) / 1e9 / peak}}


def _r(x, n=3):
    """Rounds to n significant digits (compact summary)."""
    if x is None or not isinstance(x, (int, float)) or x == 0 or not np.isfinite(x):
        return x
    return float(f"{x:.{n}g}")


def summary(line: dict) -> dict:
    """The headline figures of every section, rounded, for the end of the JSON line."""
    g = lambda d, *k: (None if d is None else (d.get(k[0]) if len(k) == 1 else g(d.get(k[0]), *k[1:])))
    out = {"c1": {"value": _r(line["value"]), "e2e": _r(line["e2e"]["value"]),
                  "frac_alg": _r(line["roofline"]["frac"]), "dram_frac": _r(line["roofline"].get("dram_frac")),
                  "vs_cpu": _r(line["value"] / line["cpu_baseline"]["value"]) if line.get("cpu_baseline") else None,
                  "vs_cpu_1core": _r(line["value"] / line["cpu_baseline_single_thread"]["value"])
                  if line.get("cpu_baseline_single_thread") else None}}
    par = line.get("parity")
    if par:
        out["parity"] = {"steps": par["steps"], "bitdiff_kernel_order_100": par["kernel_order_cells_differing_after_100"],
                         "rel": _r(par["rel_linf"], 2), "rel_cfl": _r(par["rel_linf_cfl_rows"], 2),
                         "rel_stable": _r(par["rel_linf_stable_rows_margin8"], 2),
                         "rel_sin02": _r(par["rel_linf_sin_ge_0.2"], 2)}
    cs = line.get("cpu_semantics")
    if cs:
        out["cpu_sem"] = {"value": _r(cs["f32x2"]["value"]), "frac16": _r(cs["f32x2"]["roofline"]["frac"]),
                          "frac8": _r(cs["f32x2"]["roofline"]["frac_at_8B_per_cell_step"]),
                          "f32_frac8": _r(cs["f32"]["roofline"]["frac"]), "vs_cpu_f64": _r(cs["vs_cpu_baseline"])}
    if line.get("res4096"):
        out["res4096"] = {"value": _r(line["res4096"]["value"]), "frac_alg": _r(line["res4096"]["roofline"]["frac"]),
                          "dram_frac": _r(line["res4096"]["roofline"]["dram_frac"])}
    if line.get("foam"):
        out["foam"] = {"value": _r(line["foam"]["value"]), "gbs_alg": _r(line["foam"]["algorithmic_gbs"])}
    sp = line.get("spectral")
    if sp:
        out["spectral"] = {k: _r(g(sp, k, "value")) for k in sp if isinstance(sp.get(k), dict) and "value" in sp[k]}
    for key in ("surrogate", "surrogate_hswish"):
        su = line.get(key)
        if su:
            ho = su.get("heldout_256") or {}
            out[key] = {"x_plain": _r(su["speedup_vs_plain"]), "err": _r(su["masked_rel_linf_vs_plain"], 2),
                        "train_tflops": _r((su.get("train") or {}).get("tflops")),
                        "id_err": _r(su["identity_rel_linf_vs_plain"], 2), "tc_frac": _r(su["tensor"]["frac"]),
                        "held": _r(ho.get("rel_linf"), 2), "held_id": _r(ho.get("rel_linf_identity"), 2),
                        "fail": (su.get("stats") or {}).get("failed_checks")}
    for key in ("shading", "caustics", "branched_flow", "foam_dynamics"):
        if line.get(key):
            out[key] = _r(line[key]["value"])
    ca = (line.get("caustics") or {}).get("run_and_map") or {}
    if ca.get("passes_10"):
        out["caustics_frame10_us"] = {"separate": _r(ca["passes_10"]["separate_us"]),
                                      "fused": _r(ca["passes_10"]["fused_us"])}
    return out


def main():
    args = parse()
    if args.impl == "reference":
        return run_reference(args)
    rank, world, local = dist_env()
    import torch

    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    torch.cuda.set_device(local)
    import soap_bubble_simulation_gb300 as sbs
    from soap_bubble_simulation_gb300 import _native as N
    from soap_bubble_simulation_gb300 import synthetic

    h0, c0 = synthetic.bubble_c1(RES)
    nt, np_ = h0.shape
    cells = h0.size
    sim = sbs.GPUDrainageSimulator(None, 550e-9, np_, nt)
    stream = torch.cuda.ExternalStream(sim.stream())
    flush = torch.empty(512 << 20, dtype=torch.uint8, device="cuda")

    def barrier():
        torch.cuda.synchronize()
        if world > 1:
            torch.distributed.barrier()

    # ---- device-resident throughput ------------------------------------------------------
    sim.set_thickness_array(h0)
    sim.set_concentration_array(c0)
    vols = None
    for _ in range(args.warmup):
        with torch.cuda.stream(stream):
            flush.zero_()
        vols = sim.run_checked(0.0, STEPS_PER_RUN, CHECK_EVERY)
    barrier()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    with ClockSampler(local) as clk:
        start_all = torch.cuda.Event(enable_timing=True)
        end_all = torch.cuda.Event(enable_timing=True)
        barrier()
        start_all.record(stream)
        for k in range(args.steps):
            with torch.cuda.stream(stream):
                flush.zero_()
            ev[k][0].record(stream)
            vols = sim.run_checked(0.0, STEPS_PER_RUN, CHECK_EVERY)
            ev[k][1].record(stream)
        end_all.record(stream)
        barrier()
    total_ms = start_all.elapsed_time(end_all)
    kern_ms = sum(a.elapsed_time(b) for a, b in ev)
    total_ms, kern_ms = max_over_ranks(total_ms, kern_ms)
    value = world * cells * STEPS_PER_RUN * args.steps / (total_ms / 1e3)
    kb = ctypes.c_int()
    N.call("sbs_gpu_drainage_time_blocking", sim.handle, ctypes.byref(kb))
    k_block = max(1, kb.value)
    launches = launches_per_run(k_block)
    # the dominant kernel: k-step launches; algorithmic bytes per launch = 16 B x cells x k
    step_us = kern_ms * 1e3 / (args.steps * STEPS_PER_RUN)
    launch_us = step_us * k_block
    peak, peak_kind = hbm_peak()
    achieved = BYTES_PER_CELL_STEP * cells * k_block / (launch_us * 1e-6) / 1e9
    traffic = ncu_traffic()
    vol_drift = float(abs(vols[-1] - vols[0]) / vols[0]) if vols is not None and len(vols) else None

    # ---- end to end through the C ABI with host buffers -------------------------------------
    hp = torch.from_numpy(np.ascontiguousarray(h0)).pin_memory()
    cp = torch.from_numpy(np.ascontiguousarray(c0)).pin_memory()
    ho = torch.empty_like(hp).pin_memory()
    co = torch.empty_like(cp).pin_memory()
    e2e_steps = max(1, min(args.steps, 2))

    def e2e_once():
        N.call("sbs_drainage_set_thickness", sim.handle, ctypes.c_void_p(hp.data_ptr()), cells, N.MEM_HOST)
        N.call("sbs_drainage_set_concentration", sim.handle, ctypes.c_void_p(cp.data_ptr()), cells, N.MEM_HOST)
        v = np.zeros(STEPS_PER_RUN // CHECK_EVERY)
        N.call("sbs_drainage_run_checked", sim.handle, 0.0, STEPS_PER_RUN, CHECK_EVERY, N.dptr(v))
        N.call("sbs_drainage_get_thickness_field", sim.handle, ctypes.c_void_p(ho.data_ptr()), cells, N.MEM_HOST)
        N.call("sbs_drainage_get_concentration_field", sim.handle, ctypes.c_void_p(co.data_ptr()), cells,
               N.MEM_HOST)
        return v

    e2e_once()
    barrier()
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        e2e_once()
    barrier()
    e2e_s = time.perf_counter() - t0
    (e2e_s,) = max_over_ranks(e2e_s)
    e2e_value = world * cells * STEPS_PER_RUN * e2e_steps / e2e_s

    surrogate = foam = spectral = small = shade = caus = bflow = fdyn = cpu_sem = big = None
    if not args.skip_aux:
        cpu_sem = cpu_semantics_section(sbs, torch, h0, peak,
                                         min(args.cpu_seconds, 10.0) if rank == 0 and world == 1 else 0.5)
        big = res4096_section(sbs, synthetic, torch, peak)
        small = c0_section(sbs, synthetic, torch)
        shade = shade_section(sbs, torch)
        caus = caustics_section(sbs, synthetic, torch, h0, c0)
        bflow = branched_section(sbs, synthetic, torch)
        surrogate = surrogate_section(sbs, synthetic, h0, c0, torch)
        foam = foam_section(sbs, synthetic, torch)
        spectral = spectral_section(sbs, synthetic, torch)
        if rank == 0 and world == 1:
            fdyn = foam_dynamics_section(sbs, min(args.cpu_seconds, 10.0))

    base = base1 = par = None
    if rank == 0 and world == 1 and not args.skip_aux:
        base, sample = cpu_baseline(h0, c0, args.cpu_seconds, os.cpu_count() or 1)
        par = parity_section(sbs, sample, h0, c0)
        # one host core: the reference's own CPU code is single-threaded
        base1, _ = cpu_baseline(h0, c0, min(args.cpu_seconds, 6.0), 1)

    if rank == 0:
        roof = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                "traffic": traffic, "peak_kind": peak_kind, "bytes_per_launch": BYTES_PER_CELL_STEP * cells * k_block,
                "steps_per_launch": k_block, "launch_us": launch_us,
                "dram_frac": traffic / (launch_us * 1e-6) / 1e9 / peak if traffic else None,
                "kernel": f"wtb_wgsl_kernel<{k_block}> (temporally blocked WGSL step)",
                "note": "algorithmic bytes: 16 B per cell-step; temporal blocking keeps k steps on chip, so achieved "
                        "can exceed the copy peak; traffic is ncu DRAM bytes per launch (L2 holds part of the 128 MB "
                        "working set at this size; see res4096 for a size L2 cannot hold)"}
        line = {
            "metric": METRIC, "value": value, "unit": "cell-steps/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": workload_config(world),
            "roofline": roof,
            "e2e": {"value": e2e_value, "unit": "cell-steps/s", "h2d_bytes_per_step": 2 * cells * 4,
                    "d2h_bytes_per_step": 2 * cells * 4 + 8 * (STEPS_PER_RUN // CHECK_EVERY)},
            "gpu_launches": args.steps * launches,
            "clocks": clk.summary(),
            "cpu_baseline": base,
            "cpu_baseline_single_thread": base1,
            "parity": par,
            "volume_rel_drift_per_run": vol_drift,
            "cpu_semantics": cpu_sem,
            "res4096": big,
            "surrogate": surrogate and surrogate["gelu"],
            "surrogate_hswish": surrogate and surrogate["hswish"],
            "foam": foam,
            "spectral": spectral,
            "c0": small,
            "shading": shade,
            "caustics": caus,
            "branched_flow": bflow,
            "foam_dynamics": fdyn,
        }
        line["summary"] = summary(line)
        print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
