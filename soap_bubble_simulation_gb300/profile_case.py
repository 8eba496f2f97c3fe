"""Runs one drainage workload for a fixed number of steps, for profilers (ncu) to attach to.

    python -m soap_bubble_simulation_gb300.profile_case --case wgsl --res 2048 --steps 20

Cases: `wgsl` (GPUDrainageSimulator semantics, h + surfactant), `cpu` (DrainageSimulator
semantics, compensated f32x2), `cpu32` (plain f32), `spectral-tc` / `spectral-fp32` (81-wavelength
spectral colour of --points seeded points, tensor-core or FP32 contraction), `surrogate-fused` /
`surrogate-layered` (--steps 64-pass surrogate intervals of the field, untrained seeded weights:
the same kernels and shapes as a trained network; --activation gelu or hswish), `train` (--steps
surrogate training iterations, batch 8 x 256 x 512, on 24 seeded trajectories), `foam` (the 4096-bubble foam batch, --steps
steps with the default tiles), `shade` (--steps 3840 x 2160 headless frames of the bubble
fragment shader), `caustics` (--steps caustic maps of the field after 100 WGSL passes),
`foam-dynamics` (FoamSimulator::step on an FCC foam of --bubbles bubbles: 3 steps, then --steps
steps in one call), `branched` (--steps branched-flow steps at the reference's defaults, patch
off, over a seeded 128 x 64 film). The field is the seeded smooth-mode field of
the 2048-resolution workload, built at the requested resolution. Steps launch one kernel each
(graph replay for runs of 8 or more).
"""
from __future__ import annotations

import argparse
import ctypes

from . import _native as N
from . import synthetic
from .config import SimulationConfig
from .drainage import DrainageSimulator, GPUDrainageSimulator, _Handle


def main(argv=None) -> None:
    p = argparse.ArgumentParser()
    p.add_argument("--case", default="wgsl",
                   choices=["wgsl", "cpu", "cpu32", "spectral-tc", "spectral-fp32", "surrogate-fused", "surrogate-layered",
                            "train",
                            "foam", "shade", "caustics", "foam-dynamics", "branched"])
    p.add_argument("--points", type=int, default=1 << 20, help="spectral cases: number of points")
    p.add_argument("--res", type=int, default=2048)
    p.add_argument("--steps", type=int, default=20)
    p.add_argument("--blocking", type=int, default=-1,
                   help="steps per launch, both semantics (default: library choice; 1 = single steps)")
    p.add_argument("--bubbles", type=int, default=4096, help="foam case: number of bubbles")
    p.add_argument("--activation", default="gelu", choices=["gelu", "hswish"], help="surrogate cases: activation")
    a = p.parse_args(argv)
    if a.case.startswith("spectral"):
        from .interference import spectral_rgb

        t, ci, nf = synthetic.spectral_points(a.points)
        wl = synthetic.WAVELENGTHS_81
        cmf = synthetic.spectral_cmf(wl)
        for _ in range(a.steps):
            spectral_rgb(t, ci, nf, wl, cmf, mode="tc" if a.case == "spectral-tc" else "fp32")
        print(f"ran {a.steps} spectral evaluations of {a.points} points ({a.case})")
        return
    if a.case == "shade":
        from .shading import BubbleUniform, Camera, render_frame

        u = BubbleUniform.default()
        u.set_time(2.0)
        cam = Camera(aspect=16 / 9, distance=0.06)
        for _ in range(a.steps):
            render_frame(u, cam, 3840, 2160)
        print(f"shaded {a.steps} 3840 x 2160 frames")
        return
    if a.case == "foam-dynamics":
        from .foam_dynamics import FoamSimulator, fcc_foam

        sim = FoamSimulator(*fcc_foam(a.bubbles, seed=0))
        sim.step(1e-3, 3)
        sim.step(1e-3, a.steps)
        print(f"stepped a {a.bubbles}-bubble foam {a.steps + 3} times ({sim.connection_count()} connections)")
        return
    if a.case == "branched":
        import numpy as np

        from .branched import BranchedFlowParams, branched_flow_step, generate_scatterers

        bp = BranchedFlowParams.default()
        bp.patch_enabled = 0
        th = (synthetic.smooth_modes(64, 128, seed=3) * 2e4).astype(np.float32)
        sc = generate_scatterers(bp, time=1.5)
        tex = np.zeros((bp.tex_height, bp.tex_width), np.uint32)
        for _ in range(a.steps):
            tex = branched_flow_step(bp, th, sc, tex)
        print(f"ran {a.steps} branched-flow steps")
        return
    if a.case == "foam":
        from .foam import FoamDrainage

        res, rad = synthetic.foam_bubbles(a.bubbles)
        foam = FoamDrainage(res, rad)
        hs = synthetic.foam_fields(res)
        for b in range(len(res)):
            foam.set_thickness(b, hs[b])
        foam.run(a.steps)
        foam.close()
        print(f"ran {a.steps} foam steps of {len(res)} bubbles")
        return
    h, c = synthetic.bubble_c1(a.res)
    if a.case == "train":
        from .surrogate import DrainageSurrogate, field_params

        s = DrainageSurrogate(seed=7, activation=a.activation)
        for hh, cc, visc, rad in synthetic.surrogate_trajectories(24):
            s.add_trajectory(hh, cc, field_params(256, 512, viscosity=visc, bubble_radius=rad), pairs=4)
        s.train(16, a.steps, batch=8, lr=2e-3, seed=5)
        s.close()
        print(f"ran {a.steps} training iterations (batch 8 x 256 x 512, {a.activation})")
        return
    if a.case.startswith("surrogate"):
        from .surrogate import DrainageSurrogate, field_params

        s = DrainageSurrogate(seed=7, activation=a.activation)
        sim = GPUDrainageSimulator(None, 550e-9, 2 * a.res, a.res)
        sim.update_params(field_params(a.res, 2 * a.res, bubble_radius=0.025))
        sim.set_thickness_array(h)
        sim.set_concentration_array(c)
        for _ in range(a.steps):
            s.advance(sim, mode="fused" if a.case == "surrogate-fused" else "layered")
        s.close()
        sim.close()
        print(f"ran {a.steps} surrogate intervals ({a.case}, {a.activation}) at resolution {a.res}")
        return
    if a.case == "caustics":
        sim = GPUDrainageSimulator(None, 550e-9, 2 * a.res, a.res)
        sim.set_thickness_array(h)
        sim.set_concentration_array(c)
        sim.run(100)
        for _ in range(a.steps):
            sim.caustic_map()
        sim.close()
        print(f"ran {a.steps} caustic maps at resolution {a.res}")
        return
    if a.case == "wgsl":
        sim = GPUDrainageSimulator(None, 550e-9, 2 * a.res, a.res)
        if a.blocking >= 0:
            N.call("sbs_gpu_drainage_set_time_blocking", sim.handle, a.blocking)
        sim.set_thickness_array(h)
        sim.set_concentration_array(c)
        sim.run(a.steps)
    else:
        cfg = SimulationConfig()
        cfg.resolution = a.res
        cc = cfg.to_c()
        hh = ctypes.c_void_p()
        prec = N.DRAIN_F32X2 if a.case == "cpu" else N.DRAIN_F32
        N.call("sbs_drainage_create_ex", ctypes.byref(cc), prec, ctypes.byref(hh))
        sim = DrainageSimulator.__new__(DrainageSimulator)
        _Handle.__init__(sim)
        sim._h = hh
        if a.blocking >= 0:
            N.call("sbs_drainage_set_time_blocking", sim.handle, a.blocking)
        sim.set_thickness_array(h)
        sim.step_n(cfg.dt, a.steps)
    sim.close()
    print(f"ran {a.steps} steps of case {a.case} at resolution {a.res}")


if __name__ == "__main__":
    main()
