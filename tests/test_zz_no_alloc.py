"""The no-allocation film volume (sbs_film_volume_device_noalloc) against the allocating one.

Some callers cannot let a library allocate GPU memory while they run (an engine that has handed
the device's memory to its own pool, a real-time loop that cannot take an allocation's stall).
For them libsbs keeps the volume reduction's scratch in one fixed device array. This test calls
the new entry point through the C ABI twice in a row, on two different fields, and checks each
result against sbs_film_volume_device within the 1e-12 relative tolerance the volume tests use.
It also checks that a grid beyond the stated 16384-row limit is refused. This file sorts last,
so a run that stops at the first failure has already run every other test.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def volumes(sbs, fn, field):
    out = ctypes.c_double()
    sbs._native.call(fn, ctypes.c_void_p(field.ptr), field.num_theta, field.num_phi, field.pitch, 0.025,
                     ctypes.byref(out), ctypes.c_void_p(field.stream))
    return out.value


def test_noalloc_volume_matches_allocating_entry_point(sbs):
    from soap_bubble_simulation_gb300 import synthetic

    fields = []
    for k, (W, H) in enumerate([(4096, 2048), (130, 33)]):
        sim = sbs.GPUDrainageSimulator(None, 500e-9, W, H)
        sim.set_thickness_array(synthetic.smooth_modes(H, W, seed=k + 11).astype(np.float32))
        fields.append((sim, sim.current_thickness_buffer()))
    for call in range(2):  # two calls in a row: the shared array's old contents must not leak
        for sim, f in fields:
            want = volumes(sbs, "sbs_film_volume_device", f)
            got = volumes(sbs, "sbs_film_volume_device_noalloc", f)
            assert got == pytest.approx(want, rel=1e-12), (call, got, want)
            assert got > 0


def test_noalloc_volume_rejects_grids_beyond_its_limit(sbs):
    sim = sbs.GPUDrainageSimulator(None, 500e-9, 128, 64)
    f = sim.current_thickness_buffer()
    out = ctypes.c_double()
    rc = sbs._native.lib().sbs_film_volume_device_noalloc(ctypes.c_void_p(f.ptr), 16385, 128, f.pitch, 0.025,
                                                          ctypes.byref(out), None)
    assert rc == sbs._native.SBS_E_INVALID
    assert "16384" in sbs._native.last_error()
