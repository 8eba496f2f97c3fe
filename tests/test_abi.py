"""The C-ABI library loads, and exports exactly what include/sbs.h declares. No compute calls:
on a machine without a GPU the library must refuse work with SBS_E_CUDA, never compute on the CPU."""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "sbs.h")


def declared_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"^\s*(?:int|const char \*)\s*(sbs_\w+)\s*\(", text, flags=re.M)))


@pytest.fixture(scope="module")
def lib():
    from soap_bubble_simulation_gb300 import _native

    if not os.path.exists(_native.LIB_PATH):
        from soap_bubble_simulation_gb300 import build

        build.build()
    return _native.lib()


def test_header_declares_functions():
    names = declared_functions()
    assert len(names) >= 50
    assert "sbs_drainage_step" in names and "sbs_interference_lut_rgba8" in names


def test_every_declared_symbol_is_exported(lib):
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing


def test_binding_covers_the_header():
    from soap_bubble_simulation_gb300 import _native

    assert sorted(_native.SIGNATURES) == declared_functions()


def test_no_gpu_means_an_error_not_a_fallback(lib):
    from soap_bubble_simulation_gb300 import _native

    n = ctypes.c_int(-1)
    rc = lib.sbs_device_count(ctypes.byref(n))
    if rc == 0 and n.value > 0:
        pytest.skip("a GPU is visible here")
    cfg = _native.SbsConfig()
    assert lib.sbs_config_default(ctypes.byref(cfg)) == 0
    assert cfg.resolution == 128 and cfg.dt == 0.001
    h = ctypes.c_void_p()
    assert lib.sbs_drainage_create(ctypes.byref(cfg), ctypes.byref(h)) == _native.SBS_E_CUDA
    assert not h
    assert b"CUDA" in lib.sbs_last_error() or b"device" in lib.sbs_last_error()


def test_argument_validation_before_device(lib):
    from soap_bubble_simulation_gb300 import _native

    cfg = _native.SbsConfig()
    lib.sbs_config_default(ctypes.byref(cfg))
    cfg.resolution = 2
    h = ctypes.c_void_p()
    assert lib.sbs_drainage_create(ctypes.byref(cfg), ctypes.byref(h)) == _native.SBS_E_INVALID
    assert b"resolution" in lib.sbs_last_error()


def test_params_default_matches_reference(lib):
    from soap_bubble_simulation_gb300 import DrainageParams, _native

    p = _native.SbsDrainageParams()
    assert lib.sbs_drainage_params_default(ctypes.byref(p)) == 0
    assert DrainageParams.from_c(p) == DrainageParams(dt=p.dt, bubble_radius=p.bubble_radius,
                                                      critical_thickness=p.critical_thickness,
                                                      diffusion_coeff=p.diffusion_coeff, gamma_air=p.gamma_air,
                                                      gamma_reduction=p.gamma_reduction,
                                                      surfactant_diffusion=p.surfactant_diffusion,
                                                      marangoni_coeff=p.marangoni_coeff, gravity=p.gravity,
                                                      viscosity=p.viscosity)
    assert (p.grid_width, p.grid_height, p.marangoni_enabled) == (128, 64, 0)
    assert p.critical_thickness == pytest.approx(30e-9)
