"""Writes the oracle's regression fixtures into this folder (run from the repository root:
`python tests/golden/make_golden.py`).

The reference ships no numeric golden vectors for this path and cannot be run here (Rust + wgpu,
no toolchain), so the oracle is pinned by the reference's own known-answer unit tests and by
closed forms (tests/test_oracle_*.py). These fixtures are a different thing: small outputs of the
pinned oracle, committed so that any later change to the oracle that alters them shows up as a
failing test and has to be explained.
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))


def cases():
    import oracle as orc

    from soap_bubble_simulation_gb300 import foam_dynamics, synthetic

    out = {}
    # the RGBA8 interference LUT of interference_lut.rs (n = 1.33, intensity 1)
    out["lut_rgba8_133"] = np.asarray(orc.interference_lut_rgba8(1.33, 1.0), dtype=np.uint8)
    # DrainageSimulator semantics, f64, resolution 33, 80 steps of 10 ms (fronts active from step 50)
    sim = orc.CpuSim(resolution=33, precision="f64")
    sim.set_field(synthetic.bubble_c0(33, seed=0))
    sim.step_n(0.01, 80)
    out["drainage_cpu_f64_r33_80"] = np.asarray(sim.field(), dtype=np.float64)
    # FoamSimulator: the default cluster after 11 steps of 16 ms
    pos, rad = foam_dynamics.default_cluster()
    p = foam_dynamics.FoamPhysics.default()
    r = orc.foam_step(p, 0.016, 11, pos, rad)
    out["foam_default_11_position"] = r["position"]
    out["foam_default_11_velocity"] = r["velocity"]
    out["foam_default_11_connections"] = np.stack([r["connections"]["bubble_a"], r["connections"]["bubble_b"]], 1)
    return out


if __name__ == "__main__":
    np.savez_compressed(os.path.join(HERE, "oracle_regression.npz"), **cases())
    print("wrote", os.path.join(HERE, "oracle_regression.npz"))
