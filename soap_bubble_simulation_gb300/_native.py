"""ctypes binding of libsbs.so (include/sbs.h).

The library is the only compute path: if it is missing or cannot be loaded,
`lib()` raises and nothing falls back to the CPU.
"""
from __future__ import annotations

import ctypes as C
import os
import threading

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_build", "libsbs.so")

SBS_OK = 0
SBS_E_INVALID = -1
SBS_E_CUDA = -2
SBS_E_TIMEOUT = -3
SBS_E_NONFINITE = -4
SBS_E_NOMEM = -5
SBS_E_STATE = -6

MEM_HOST = 0
MEM_DEVICE = 1
CPU_SEMANTICS = 0
WGSL_SEMANTICS = 1
PREC_F64 = 0
PREC_F32 = 1
DRAIN_F32 = 0
DRAIN_F32X2 = 1
SPECTRAL_TC_BF16 = 0
SPECTRAL_FP32 = 1
LOOKUP_GRID = 0
LOOKUP_TEXEL = 1
NN_LAYERED = 0
NN_FUSED = 1
NN_PARAMS = 23425
NN_ACT_GELU = 0
NN_ACT_HSWISH = 1
NN_STEPS = 64
STALL_TENSOR_COMMITS = 1
STALL_GRID_BARRIER = 2

_ERR_NAMES = {
    SBS_E_INVALID: "SBS_E_INVALID",
    SBS_E_CUDA: "SBS_E_CUDA",
    SBS_E_TIMEOUT: "SBS_E_TIMEOUT",
    SBS_E_NONFINITE: "SBS_E_NONFINITE",
    SBS_E_NOMEM: "SBS_E_NOMEM",
    SBS_E_STATE: "SBS_E_STATE",
}


class SbsError(RuntimeError):
    """A libsbs call returned a negative status."""

    def __init__(self, code: int, message: str):
        super().__init__(f"{_ERR_NAMES.get(code, code)}: {message}")
        self.code = code


class SbsConfig(C.Structure):
    """sbs_config (include/sbs.h), the C mirror of SimulationConfig (config.rs:283-302)."""

    _fields_ = [
        ("diameter", C.c_double),
        ("film_thickness_nm", C.c_double),
        ("critical_thickness_nm", C.c_double),
        ("refractive_index", C.c_double),
        ("viscosity", C.c_double),
        ("surface_tension", C.c_double),
        ("density", C.c_double),
        ("surfactant_diffusion", C.c_double),
        ("surfactant_concentration", C.c_double),
        ("gravity", C.c_double),
        ("temperature", C.c_double),
        ("pressure", C.c_double),
        ("dt", C.c_double),
        ("resolution", C.c_uint32),
        ("_reserved", C.c_uint32),
    ]


class SbsDrainageParams(C.Structure):
    """sbs_drainage_params, the 64-byte DrainageParams uniform (gpu_drainage.rs:12-44)."""

    _fields_ = [
        ("dt", C.c_float),
        ("gravity", C.c_float),
        ("viscosity", C.c_float),
        ("density", C.c_float),
        ("diffusion_coeff", C.c_float),
        ("bubble_radius", C.c_float),
        ("critical_thickness", C.c_float),
        ("grid_width", C.c_uint32),
        ("grid_height", C.c_uint32),
        ("marangoni_enabled", C.c_uint32),
        ("gamma_air", C.c_float),
        ("gamma_reduction", C.c_float),
        ("surfactant_diffusion", C.c_float),
        ("marangoni_coeff", C.c_float),
        ("_padding1", C.c_uint32),
        ("_padding2", C.c_uint32),
    ]


assert C.sizeof(SbsDrainageParams) == 64

_P = C.c_void_p
_D = C.c_double
_F = C.c_float
_U32 = C.c_uint32
_SZ = C.c_size_t
_I = C.c_int
_DP = C.POINTER(C.c_double)
_FP = C.POINTER(C.c_float)
_U32P = C.POINTER(C.c_uint32)
_IP = C.POINTER(C.c_int)

# name -> argtypes (every function returns int unless listed in _RESTYPES)
SIGNATURES: dict[str, list] = {
    "sbs_last_error": [],
    "sbs_version": [],
    "sbs_device_count": [_IP],
    "sbs_config_default": [C.POINTER(SbsConfig)],
    "sbs_drainage_params_default": [C.POINTER(SbsDrainageParams)],
    "sbs_drainage_create": [C.POINTER(SbsConfig), C.POINTER(_P)],
    "sbs_drainage_create_ex": [C.POINTER(SbsConfig), _I, C.POINTER(_P)],
    "sbs_drainage_precision": [_P, _IP],
    "sbs_gpu_drainage_create": [_F, _U32, _U32, C.POINTER(_P)],
    "sbs_drainage_destroy": [_P],
    "sbs_drainage_semantics": [_P, _IP],
    "sbs_drainage_grid_size": [_P, _U32P, _U32P],
    "sbs_drainage_step": [_P, _D],
    "sbs_drainage_step_n": [_P, _D, _U32],
    "sbs_gpu_drainage_step": [_P, _F],
    "sbs_gpu_drainage_run": [_P, _U32],
    "sbs_drainage_run_checked": [_P, _D, _U32, _U32, _DP],
    "sbs_drainage_set_thickness": [_P, _P, _SZ, _I],
    "sbs_drainage_get_thickness_field": [_P, _P, _SZ, _I],
    "sbs_drainage_set_concentration": [_P, _P, _SZ, _I],
    "sbs_drainage_get_concentration_field": [_P, _P, _SZ, _I],
    "sbs_drainage_set_thickness_f64": [_P, _DP, _SZ],
    "sbs_drainage_get_thickness_field_f64": [_P, _DP, _SZ],
    "sbs_drainage_thickness_device": [_P, _I, C.POINTER(_P), C.POINTER(_SZ)],
    "sbs_drainage_concentration_device": [_P, _I, C.POINTER(_P), C.POINTER(_SZ)],
    "sbs_drainage_stream": [_P, C.POINTER(_P)],
    "sbs_drainage_get_thickness": [_P, _D, _D, _DP],
    "sbs_drainage_query_batch": [_P, _P, _P, _P, _SZ, _I],
    "sbs_drainage_current_time": [_P, _DP],
    "sbs_drainage_has_critical_region": [_P, _IP],
    "sbs_drainage_critical_thickness": [_P, _DP],
    "sbs_drainage_min_max": [_P, _DP, _DP],
    "sbs_drainage_film_volume": [_P, _DP],
    "sbs_drainage_reset": [_P, _D],
    "sbs_drainage_set_marginal_regeneration": [_P, _I],
    "sbs_drainage_marginal_regeneration_enabled": [_P, _IP],
    "sbs_drainage_set_tfe_thickness_ratio": [_P, _D],
    "sbs_drainage_tfe_thickness_ratio": [_P, _DP],
    "sbs_drainage_active_tfe_count": [_P, _U32P],
    "sbs_gpu_drainage_update_params": [_P, C.POINTER(SbsDrainageParams)],
    "sbs_gpu_drainage_params": [_P, C.POINTER(SbsDrainageParams)],
    "sbs_gpu_drainage_set_dt": [_P, _F],
    "sbs_gpu_drainage_set_physics": [_P, _F, _F, _F, _F],
    "sbs_gpu_drainage_set_bubble_radius": [_P, _F],
    "sbs_gpu_drainage_set_marangoni_enabled": [_P, _I],
    "sbs_gpu_drainage_set_marangoni_params": [_P, _F, _F, _F, _F],
    "sbs_gpu_drainage_set_time_blocking": [_P, _I],
    "sbs_gpu_drainage_time_blocking": [_P, _IP],
    "sbs_set_wait_limit": [C.c_uint64],
    "sbs_wait_limit": [C.POINTER(C.c_uint64)],
    "sbs_set_stall_injection": [_I],
    "sbs_drainage_set_time_blocking": [_P, _I],
    "sbs_drainage_time_blocking": [_P, _IP],
    "sbs_gpu_drainage_set_enabled": [_P, _I],
    "sbs_gpu_drainage_set_time_scale": [_P, _F],
    "sbs_gpu_drainage_set_steps_per_frame": [_P, _U32],
    "sbs_film_volume_device": [_P, _U32, _U32, _SZ, _D, _DP, _P],
    "sbs_film_volume_device_noalloc": [_P, _U32, _U32, _SZ, _D, _DP, _P],
    "sbs_interference_color_batch": [_D, _DP, _P, _P, _SZ, _I, _I, _P, _I, _P],
    "sbs_interference_terms_batch": [_D, _D, _P, _P, _SZ, _P, _I, _P],
    "sbs_optical_path_batch": [_D, _P, _P, _P, _SZ, _P, _I, _P],
    "sbs_phase_difference_batch": [_P, _P, _SZ, _P, _I, _P],
    "sbs_lut1d_build": [_D, _DP, _D, _D, _U32, _D, _P, _I, _P],
    "sbs_lut2d_build": [_D, _DP, _D, _D, _U32, _U32, _P, _I, _P],
    "sbs_interference_lut_rgba8": [_F, _F, _P, _I, _P],
    "sbs_schlick_rgb_batch": [_F, _FP, _P, _P, _SZ, _P, _I, _P],
    "sbs_lut_rgba8_lookup_batch": [_P, _U32, _U32, _F, _F, _I, _P, _P, _SZ, _P, _I, _P],
    "sbs_lut2d_lookup_batch": [_P, _U32, _U32, _D, _D, _P, _P, _SZ, _P, _I, _P],
    "sbs_foam_create": [_U32, _P, _P, C.POINTER(SbsDrainageParams), C.POINTER(_P)],
    "sbs_foam_destroy": [_P],
    "sbs_foam_total_cells": [_P, C.POINTER(C.c_uint64)],
    "sbs_foam_set_thickness": [_P, _U32, _P, _SZ, _I],
    "sbs_foam_get_thickness": [_P, _U32, _P, _SZ, _I],
    "sbs_foam_set_concentration": [_P, _U32, _P, _SZ, _I],
    "sbs_foam_get_concentration": [_P, _U32, _P, _SZ, _I],
    "sbs_foam_run": [_P, _U32],
    "sbs_foam_set_tiles": [_P, _U32, _U32],
    "sbs_foam_autotune": [_P, _U32, _U32P, _U32P],
    "sbs_foam_stream": [_P, C.POINTER(_P)],
    "sbs_spectral_rgb": [_P, _P, _P, _SZ, _P, _U32, _P, _I, _P, _I, _P],
    "sbs_bubble_uniform_default": [_P],
    "sbs_shade_fragments": [_P, _P, _P, _P, _SZ, _P, _P, _P, _I, _P],
    "sbs_shade_frame": [_P, _P, _P, _F, _P, _P, _U32, _U32, _P, _P, _I, _P],
    "sbs_caustic_params_default": [_P],
    "sbs_caustics": [_P, _P, _SZ, _P, _I, _P],
    "sbs_gpu_drainage_caustics": [_P, _P, _I, _P, _I],
    "sbs_gpu_drainage_run_caustics": [_P, C.c_uint32, _P, _P, _I],
    "sbs_gpu_drainage_step_caustics": [_P, C.c_float, _P, _P, _I],
    "sbs_branched_params_default": [_P],
    "sbs_branched_scatterers": [_P, _U32, _F, _P],
    "sbs_branched_flow": [_P, _P, _U32, _U32, _SZ, _P, _P, _I, _I, _P],
    "sbs_foam_physics_default": [_P],
    "sbs_foam_sim_create": [_U32, _P, _P, _P, _P, C.POINTER(_P)],
    "sbs_foam_sim_destroy": [_P],
    "sbs_foam_sim_set_physics": [_P, _P],
    "sbs_foam_sim_step": [_P, _F, _U32],
    "sbs_foam_sim_counts": [_P, _P, _P],
    "sbs_foam_sim_get_state": [_P, _P, _P, _P, _P, _P, _I],
    "sbs_foam_sim_set_state": [_P, _P, _P, _P, _P, _I],
    "sbs_foam_sim_forces": [_P, _P, _I],
    "sbs_foam_sim_connections": [_P, _P, _U32, _P],
    "sbs_foam_sim_couple_thickness": [_P, _P],
    "sbs_drainage_vertex_colors": [_P, _P, _SZ, _P, _U32, _U32, _D, _D, _P, _I],
    "sbs_surrogate_create": [C.c_uint64, C.POINTER(_P)],
    "sbs_surrogate_destroy": [_P],
    "sbs_surrogate_set_params": [_P, _P, _SZ],
    "sbs_surrogate_get_params": [_P, _P, _SZ],
    "sbs_surrogate_set_activation": [_P, _I],
    "sbs_surrogate_get_activation": [_P, _P],
    "sbs_surrogate_features": [_P, _U32, _P, _P, _P, _P, _I],
    "sbs_surrogate_forward": [_P, _U32, _P, _P, _P, _P, _I, _I],
    "sbs_surrogate_loss_grad": [_P, _U32, _P, _P, _P, _P, _DP, _P],
    "sbs_surrogate_add_trajectory": [_P, _P, _P, C.POINTER(SbsDrainageParams), _U32, _U32],
    "sbs_surrogate_num_trajectories": [_P, _U32P],
    "sbs_surrogate_clear_data": [_P],
    "sbs_surrogate_train": [_P, _U32, _U32, _U32, _F, C.c_uint64, _P],
    "sbs_surrogate_evaluate": [_P, _U32, _U32, _I, _P],
    "sbs_surrogate_advance": [_P, _P, _I],
    "sbs_surrogate_rollout": [_P, _P, _U32, _U32, _D, _I, _P],
    "sbs_surrogate_masked_error": [_P, _P, _U32, _U32, _I, _DP],
    "sbs_surrogate_stream": [_P, C.POINTER(_P)],
}
_RESTYPES = {"sbs_last_error": C.c_char_p, "sbs_version": C.c_char_p}

_lock = threading.Lock()
_lib: C.CDLL | None = None


def lib() -> C.CDLL:
    """Loads libsbs.so once. Raises ImportError if it has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    with _lock:
        if _lib is not None:
            return _lib
        if not os.path.exists(LIB_PATH):
            raise ImportError(
                f"libsbs.so not found at {LIB_PATH}; build it with "
                "`python -c 'import __graft_entry__ as g; g.build()'` (needs nvcc)"
            )
        L = C.CDLL(LIB_PATH)
        for name, args in SIGNATURES.items():
            fn = getattr(L, name)
            fn.argtypes = args
            fn.restype = _RESTYPES.get(name, C.c_int)
        _lib = L
        return L


def last_error() -> str:
    msg = lib().sbs_last_error()
    return msg.decode() if msg else ""


def check(rc: int) -> None:
    if rc != SBS_OK:
        raise SbsError(rc, last_error())


def call(name: str, *args) -> None:
    check(getattr(lib(), name)(*args))


def ptr(a) -> C.c_void_p:
    """Address of a C-contiguous numpy array (or None)."""
    if a is None:
        return C.c_void_p(None)
    if not a.flags["C_CONTIGUOUS"]:
        raise ValueError("array must be C-contiguous")
    return C.c_void_p(a.ctypes.data)


def dptr(a) -> C.POINTER(C.c_double):
    return a.ctypes.data_as(_DP)


def exported_symbols() -> list[str]:
    return list(SIGNATURES)
