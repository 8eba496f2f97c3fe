"""ctypes binding of the parity oracle (oracle/_build/liboracle.so).

Test infrastructure: only tests/, __graft_entry__.smoke() and bench.py's CPU
baseline legs import this module. See oracle.h for what each function
restates and how the oracle is pinned.
"""
from __future__ import annotations

import ctypes as C
import os
import sys

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
if _HERE not in sys.path:
    sys.path.insert(0, _HERE)
import build_oracle  # noqa: E402

_lib = None

_P = C.c_void_p
_D = C.c_double
_F = C.c_float
_U32 = C.c_uint32
_SZ = C.c_size_t
_I = C.c_int


class OrcSimParams(C.Structure):
    _fields_ = [
        ("resolution", C.c_uint32),
        ("diameter", C.c_double),
        ("film_thickness_nm", C.c_double),
        ("critical_thickness_nm", C.c_double),
        ("density", C.c_double),
        ("gravity", C.c_double),
        ("viscosity", C.c_double),
        ("surfactant_diffusion", C.c_double),
    ]


class OrcWgslParams(C.Structure):
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


_SIGS = {
    "orc_sim_new": ([C.POINTER(OrcSimParams), _I, _I], _P),
    "orc_sim_free": ([_P], None),
    "orc_sim_num_theta": ([_P], _U32),
    "orc_sim_num_phi": ([_P], _U32),
    "orc_sim_set_field": ([_P, _P], None),
    "orc_sim_get_field": ([_P, _P], None),
    "orc_sim_step": ([_P, _D], None),
    "orc_sim_step_n": ([_P, _D, _U32], None),
    "orc_sim_get_thickness": ([_P, _D, _D], _D),
    "orc_sim_current_time": ([_P], _D),
    "orc_sim_has_critical_region": ([_P], _I),
    "orc_sim_min_thickness": ([_P], _D),
    "orc_fix_ring_mean": ([_P, C.c_size_t, C.c_uint32], _D),
    "orc_sim_max_thickness": ([_P], _D),
    "orc_sim_reset": ([_P, _D], None),
    "orc_sim_set_marginal_regeneration": ([_P, _I], None),
    "orc_sim_set_tfe_thickness_ratio": ([_P, _D], None),
    "orc_sim_tfe_thickness_ratio": ([_P], _D),
    "orc_sim_active_tfe_count": ([_P], _U32),
    "orc_sim_get_fronts": ([_P, _P, _U32], _U32),
    "orc_wgsl_run": ([C.POINTER(OrcWgslParams), _I, _P, _P, _P, _P, _U32, _I], None),
    "orc_film_volume_f64": ([_P, _U32, _U32, _D], _D),
    "orc_film_volume_f32": ([_P, _U32, _U32, _D], _D),
    "orc_transmission_angle_cos": ([_D, _D], _D),
    "orc_optical_path_difference": ([_D, _D, _D, _D], _D),
    "orc_phase_difference": ([_D, _D], _D),
    "orc_fresnel": ([_D, _D, _P], None),
    "orc_reflected_intensity": ([_D, _D, _D, _D], _D),
    "orc_interference_color": ([_D, _P, _D, _D, _I, _P], None),
    "orc_interference_color_batch": ([_D, _P, _P, _P, _SZ, _I, _P], None),
    "orc_lut1d": ([_D, _P, _D, _D, _U32, _D, _P], None),
    "orc_lut2d": ([_D, _P, _D, _D, _U32, _U32, _P], None),
    "orc_interference_lut_rgba8": ([_F, _F, _P], None),
    "orc_thin_film_interference7": ([_F, _F, _F, _F, _P], None),
    "orc_lut_snells_law": ([_F, _F], _F),
    "orc_lut_fresnel_unpolarized": ([_F, _F, _F, _F], _F),
    "orc_schlick_interference": ([_F, _F, _F, _F], _F),
    "orc_lut_rgba8_sample": ([_P, _U32, _U32, _F, _F, _F, _F, _P], None),
    "orc_lut2d_lookup": ([_P, _U32, _U32, _D, _D, _D, _D, _P], None),
    "orc_vertex_colors": ([_P, _U32, _U32, _P, _SZ, _P, _U32, _U32, _D, _D, _P], None),
    "orc_spectral_rgb": ([_P, _P, _P, _SZ, _P, _U32, _P, _P], None),
    "orc_nn_features": ([_P, _P, C.POINTER(OrcWgslParams), _P], None),
    "orc_nn_kout": ([C.POINTER(OrcWgslParams)], _F),
    "orc_nn_forward": ([_P, _U32, _U32, _U32, _P, _P, _I], None),
    "orc_nn_loss_grad": ([_P, _U32, _U32, _U32, _P, _P, _P, _I], _D),
    "orc_nn_apply": ([_P, _P, _U32, _U32, _F, _P], None),
    "orc_acos_as": ([_F], _F),
    "orc_atan2_as": ([_F, _F], _F),
    "orc_exp_cw": ([_F], _F),
    "orc_branched_scatterers": ([_P, _U32, _F, _P], None),
    "orc_branched_flow": ([_P, _P, _U32, _U32, C.c_size_t, _P, _P, _I], None),
    "orc_pow15": ([_F], _F),
    "orc_foam_forces": ([_P, _U32, _P, _P, _P, _P, _P], None),
    "orc_foam_forces_subset": ([_P, _U32, _P, _P, _P, _P, _P, _U32, _P], None),
    "orc_foam_step": ([_P, _F, _U32, _U32, _P, _P, _P, _P, _P, _P, _P, _U32, _P], _U32),
    "orc_caustics": ([_P, _P, C.c_size_t, _P], None),
    "orc_simplex3": ([_F, _F, _F], _F),
    "orc_film_thickness": ([_P, _F, _F, _F], _F),
    "orc_shade_fragments": ([_P, _P, _P, _P, C.c_size_t, _P, _P, _P], None),
    "orc_shade_frame": ([_P, _P, _P, _F, _P, _P, _U32, _U32, _P, _P], _I),
    "orc_nn_gelu": ([_F], _F),
    "orc_nn_gelu_grad": ([_F], _F),
    "orc_nn_hswish": ([_F], _F),
    "orc_nn_hswish_grad": ([_F], _F),
    "orc_nn_set_exact": ([_I], None),
}


def lib():
    global _lib
    if _lib is None:
        path = build_oracle.build()
        L = C.CDLL(path)
        for name, (args, res) in _SIGS.items():
            fn = getattr(L, name)
            fn.argtypes = args
            fn.restype = res
        _lib = L
    return _lib


def _p(a: np.ndarray) -> C.c_void_p:
    assert a.flags["C_CONTIGUOUS"]
    return C.c_void_p(a.ctypes.data)


class CpuSim:
    """DrainageSimulator restatement (drainage.rs:212-614). precision 'f64' (faithful), 'f32k'
    (the CUDA kernel's plain f32 operation order) or 'f32x2' (its compensated hi + lo order)."""

    def __init__(self, resolution=128, diameter=0.05, film_thickness_nm=500.0, critical_thickness_nm=10.0,
                 density=1000.0, gravity=9.81, viscosity=0.001, surfactant_diffusion=1e-9, precision="f64",
                 threads=1):
        p = OrcSimParams(resolution, diameter, film_thickness_nm, critical_thickness_nm, density, gravity, viscosity,
                         surfactant_diffusion)
        mode = {"f64": 0, "f32k": 1, "f32x2": 2}[precision]
        self._h = lib().orc_sim_new(C.byref(p), mode, int(threads))
        if not self._h:
            raise ValueError("bad oracle parameters")
        self.nt = lib().orc_sim_num_theta(self._h)
        self.np = lib().orc_sim_num_phi(self._h)

    def __del__(self):
        if getattr(self, "_h", None):
            lib().orc_sim_free(self._h)
            self._h = None

    def set_field(self, h):
        a = np.ascontiguousarray(h, dtype=np.float64).reshape(-1)
        assert a.size == self.nt * self.np
        lib().orc_sim_set_field(self._h, _p(a))

    def field(self) -> np.ndarray:
        a = np.empty(self.nt * self.np, dtype=np.float64)
        lib().orc_sim_get_field(self._h, _p(a))
        return a.reshape(self.nt, self.np)

    def step(self, dt):
        lib().orc_sim_step(self._h, float(dt))

    def step_n(self, dt, n):
        lib().orc_sim_step_n(self._h, float(dt), int(n))

    def get_thickness(self, theta, phi):
        return lib().orc_sim_get_thickness(self._h, float(theta), float(phi))

    def current_time(self):
        return lib().orc_sim_current_time(self._h)

    def has_critical_region(self):
        return bool(lib().orc_sim_has_critical_region(self._h))

    def min_thickness(self):
        return lib().orc_sim_min_thickness(self._h)

    def max_thickness(self):
        return lib().orc_sim_max_thickness(self._h)

    def reset(self, h0):
        lib().orc_sim_reset(self._h, float(h0))

    def set_marginal_regeneration(self, en):
        lib().orc_sim_set_marginal_regeneration(self._h, 1 if en else 0)

    def set_tfe_thickness_ratio(self, r):
        lib().orc_sim_set_tfe_thickness_ratio(self._h, float(r))

    def tfe_thickness_ratio(self):
        return lib().orc_sim_tfe_thickness_ratio(self._h)

    def active_tfe_count(self):
        return lib().orc_sim_active_tfe_count(self._h)

    def fronts(self) -> np.ndarray:
        out = np.zeros((8, 4), dtype=np.float64)
        n = lib().orc_sim_get_fronts(self._h, _p(out), 8)
        return out[:n]


def wgsl_params(**kw) -> OrcWgslParams:
    """DrainageParams::default (gpu_drainage.rs:46-68) with overrides."""
    d = dict(dt=0.001, gravity=9.81, viscosity=0.001, density=1000.0, diffusion_coeff=1e-9, bubble_radius=0.025,
             critical_thickness=30e-9, grid_width=128, grid_height=64, marangoni_enabled=0, gamma_air=0.072,
             gamma_reduction=0.045, surfactant_diffusion=1e-9, marangoni_coeff=0.01, _padding1=0, _padding2=0)
    d.update(kw)
    p = OrcWgslParams()
    for k, v in d.items():
        setattr(p, k, v)
    return p


def wgsl_run(params: OrcWgslParams, h, c, passes: int, mode: str = "wgsl", threads: int = 0):
    """drainage.wgsl passes; mode 'wgsl' (its own op order) or 'kernel' (CUDA op order)."""
    h = np.ascontiguousarray(h, dtype=np.float32)
    c = np.ascontiguousarray(c, dtype=np.float32)
    ho = np.empty_like(h)
    co = np.empty_like(c)
    lib().orc_wgsl_run(C.byref(params), 0 if mode == "wgsl" else 1, _p(h), _p(c), _p(ho), _p(co), int(passes),
                       int(threads))
    return ho, co


def film_volume(h, radius: float) -> float:
    a = np.ascontiguousarray(h)
    nt, np_ = a.shape
    if a.dtype == np.float32:
        return lib().orc_film_volume_f32(_p(a), nt, np_, float(radius))
    a = np.ascontiguousarray(a, dtype=np.float64)
    return lib().orc_film_volume_f64(_p(a), nt, np_, float(radius))


def transmission_angle_cos(n, ci):
    return lib().orc_transmission_angle_cos(float(n), float(ci))


def optical_path_difference(n, t, ct, wl):
    return lib().orc_optical_path_difference(float(n), float(t), float(ct), float(wl))


def phase_difference(opd, wl):
    return lib().orc_phase_difference(float(opd), float(wl))


def fresnel(n, ci):
    out = np.zeros(3)
    lib().orc_fresnel(float(n), float(ci), _p(out))
    return out


def reflected_intensity(n, t, ci, wl):
    return lib().orc_reflected_intensity(float(n), float(t), float(ci), float(wl))


def interference_color(n, t, ci, gamma=True, wl=(650.0, 532.0, 450.0)):
    w = np.asarray(wl, dtype=np.float64)
    out = np.zeros(3)
    lib().orc_interference_color(float(n), _p(w), float(t), float(ci), 1 if gamma else 0, _p(out))
    return out


def interference_color_batch(n, t, ci, gamma=True, wl=(650.0, 532.0, 450.0)):
    w = np.asarray(wl, dtype=np.float64)
    t = np.ascontiguousarray(t, dtype=np.float64).reshape(-1)
    ci = np.ascontiguousarray(ci, dtype=np.float64).reshape(-1)
    out = np.zeros((t.size, 3))
    lib().orc_interference_color_batch(float(n), _p(w), _p(t), _p(ci), t.size, 1 if gamma else 0, _p(out))
    return out


def lut1d(n, tmin, tmax, count, ci, wl=(650.0, 532.0, 450.0)):
    w = np.asarray(wl, dtype=np.float64)
    out = np.zeros((count, 3))
    lib().orc_lut1d(float(n), _p(w), float(tmin), float(tmax), int(count), float(ci), _p(out))
    return out


def lut2d(n, tmin, tmax, T, A, wl=(650.0, 532.0, 450.0)):
    w = np.asarray(wl, dtype=np.float64)
    out = np.zeros((T, A, 3))
    lib().orc_lut2d(float(n), _p(w), float(tmin), float(tmax), int(T), int(A), _p(out))
    return out


def interference_lut_rgba8(n, intensity):
    out = np.zeros(64 * 256 * 4, dtype=np.uint8)
    lib().orc_interference_lut_rgba8(float(n), float(intensity), _p(out))
    return out


def thin_film_interference7(t, ci, n, intensity):
    out = np.zeros(3, dtype=np.float32)
    lib().orc_thin_film_interference7(float(t), float(ci), float(n), float(intensity), _p(out))
    return out


def lut_snells_law(ci, n):
    return lib().orc_lut_snells_law(float(ci), float(n))


def lut_fresnel_unpolarized(ci, ct, n1, n2):
    return lib().orc_lut_fresnel_unpolarized(float(ci), float(ct), float(n1), float(n2))


def schlick_interference(t, wl, ci, n):
    return lib().orc_schlick_interference(float(t), float(wl), float(ci), float(n))


def lut_rgba8_sample(lut, W, H, t, ci, max_nm=2000.0, intensity=1.0):
    L = np.ascontiguousarray(lut, dtype=np.uint8).reshape(-1)
    out = np.zeros(3, dtype=np.float32)
    lib().orc_lut_rgba8_sample(_p(L), int(W), int(H), float(t), float(ci), float(max_nm), float(intensity), _p(out))
    return out


def lut2d_lookup(lut, tmin, tmax, t, ci):
    L = np.ascontiguousarray(lut, dtype=np.float64)
    out = np.zeros(3)
    lib().orc_lut2d_lookup(_p(L), L.shape[0], L.shape[1], float(tmin), float(tmax), float(t), float(ci), _p(out))
    return out


def vertex_colors(field, xyz, lut, tmin, tmax):
    F = np.ascontiguousarray(field, dtype=np.float64)
    X = np.ascontiguousarray(xyz, dtype=np.float64)
    L = np.ascontiguousarray(lut, dtype=np.float64)
    out = np.zeros((X.shape[0], 3))
    lib().orc_vertex_colors(_p(F), F.shape[0], F.shape[1], _p(X), X.shape[0], _p(L), L.shape[0], L.shape[1],
                            float(tmin), float(tmax), _p(out))
    return out


def spectral_rgb(t, ci, n, wl, cmf):
    t = np.ascontiguousarray(t, dtype=np.float32)
    ci = np.ascontiguousarray(ci, dtype=np.float32)
    n = np.ascontiguousarray(n, dtype=np.float32)
    wl = np.ascontiguousarray(wl, dtype=np.float64)
    cmf = np.ascontiguousarray(cmf, dtype=np.float64)
    out = np.zeros((t.size, 3))
    lib().orc_spectral_rgb(_p(t), _p(ci), _p(n), t.size, _p(wl), wl.size, _p(cmf), _p(out))
    return out


# ---------------------------------------------------------------- drainage surrogate (include/sbs_nn.h)
NN_PARAMS = 23425
NN_NF = 16


def nn_features(h, c, params: OrcWgslParams) -> np.ndarray:
    """Features [nt][np][16] (BF16 values held in float32) of one field."""
    h = np.ascontiguousarray(h, dtype=np.float32)
    c = np.ascontiguousarray(c, dtype=np.float32)
    x = np.empty(h.shape + (NN_NF,), dtype=np.float32)
    lib().orc_nn_features(_p(h), _p(c), C.byref(params), _p(x))
    return x


def nn_kout(params: OrcWgslParams) -> float:
    return float(lib().orc_nn_kout(C.byref(params)))


NN_ACT = {"gelu": 0, "hswish": 1}  # SBS_NN_ACT_*


def nn_forward(theta, x, act: str = "gelu") -> np.ndarray:
    """Network output y [nb][nt][np] for features x [nb][nt][np][16]."""
    theta = np.ascontiguousarray(theta, dtype=np.float32)
    x = np.ascontiguousarray(x, dtype=np.float32)
    nb, nt, np_ = x.shape[:3]
    y = np.empty((nb, nt, np_), dtype=np.float32)
    lib().orc_nn_forward(_p(theta), nb, nt, np_, _p(x), _p(y), NN_ACT[act])
    return y


def nn_loss_grad(theta, x, target, act: str = "gelu"):
    theta = np.ascontiguousarray(theta, dtype=np.float32)
    x = np.ascontiguousarray(x, dtype=np.float32)
    target = np.ascontiguousarray(target, dtype=np.float32)
    nb, nt, np_ = x.shape[:3]
    g = np.empty(NN_PARAMS, dtype=np.float32)
    loss = lib().orc_nn_loss_grad(_p(theta), nb, nt, np_, _p(x), _p(target), _p(g), NN_ACT[act])
    return float(loss), g


def nn_apply(h, y, kout: float) -> np.ndarray:
    h = np.ascontiguousarray(h, dtype=np.float32)
    y = np.ascontiguousarray(y, dtype=np.float32)
    out = np.empty_like(h)
    lib().orc_nn_apply(_p(h), _p(y), h.shape[0], h.shape[1], float(kout), _p(out))
    return out


def nn_set_exact(exact: bool) -> None:
    lib().orc_nn_set_exact(1 if exact else 0)


def nn_gelu(x: float) -> float:
    return float(lib().orc_nn_gelu(float(x)))


def nn_gelu_grad(x: float) -> float:
    return float(lib().orc_nn_gelu_grad(float(x)))


def nn_hswish(x: float) -> float:
    return float(lib().orc_nn_hswish(float(x)))


def nn_hswish_grad(x: float) -> float:
    return float(lib().orc_nn_hswish_grad(float(x)))


# ---------------------------------------------------------------------- bubble fragment shader
def simplex3(x: float, y: float, z: float) -> float:
    return float(lib().orc_simplex3(float(x), float(y), float(z)))


def film_thickness(uniform, n) -> float:
    """get_film_thickness for one unit normal; uniform is a ctypes structure laid out as
    sbs_bubble_uniform."""
    return float(lib().orc_film_thickness(C.cast(C.byref(uniform), C.c_void_p), float(n[0]), float(n[1]), float(n[2])))


def shade_fragments(uniform, camera_pos, lut, normals, world_pos, branched=None) -> np.ndarray:
    nn = np.ascontiguousarray(normals, dtype=np.float32).reshape(-1, 3)
    wp = np.ascontiguousarray(world_pos, dtype=np.float32).reshape(-1, 3)
    cam = np.ascontiguousarray(camera_pos, dtype=np.float32).reshape(3)
    L = np.ascontiguousarray(lut, dtype=np.uint8)
    B = None if branched is None else np.ascontiguousarray(branched, dtype=np.uint32)
    out = np.empty((nn.shape[0], 4), dtype=np.float32)
    lib().orc_shade_fragments(C.cast(C.byref(uniform), C.c_void_p), _p(cam), _p(L), _p(B) if B is not None else None,
                              nn.shape[0], _p(nn), _p(wp), _p(out))
    return out


def shade_frame(uniform, view_proj, camera_pos, radius, lut, width, height, branched=None):
    """(rgba8 [h][w][4], linear [h][w][4]) of one headless frame."""
    vp = np.ascontiguousarray(view_proj, dtype=np.float32).reshape(16)
    cam = np.ascontiguousarray(camera_pos, dtype=np.float32).reshape(3)
    L = np.ascontiguousarray(lut, dtype=np.uint8)
    B = None if branched is None else np.ascontiguousarray(branched, dtype=np.uint32)
    rgba8 = np.empty((height, width, 4), dtype=np.uint8)
    lin = np.empty((height, width, 4), dtype=np.float32)
    rc = lib().orc_shade_frame(C.cast(C.byref(uniform), C.c_void_p), _p(vp), _p(cam), float(radius), _p(L),
                               _p(B) if B is not None else None, int(width), int(height), _p(rgba8), _p(lin))
    if rc != 0:
        raise ValueError("singular view_proj")
    return rgba8, lin


# ---------------------------------------------------------------------- caustics
def caustics(params, h) -> np.ndarray:
    """Caustic map of a [grid_height][grid_width] float32 field; params a ctypes structure laid out as
    sbs_caustic_params."""
    h = np.ascontiguousarray(h, dtype=np.float32)
    out = np.empty((params.grid_height, params.grid_width), dtype=np.float32)
    lib().orc_caustics(C.cast(C.byref(params), C.c_void_p), _p(h), h.shape[1], _p(out))
    return out


# ---------------------------------------------------------------------- branched flow
def acos_as(x: float) -> float:
    return float(lib().orc_acos_as(float(x)))


def atan2_as(y: float, x: float) -> float:
    return float(lib().orc_atan2_as(float(y), float(x)))


def exp_cw(x: float) -> float:
    return float(lib().orc_exp_cw(float(x)))


def branched_scatterers(params, num: int, time: float) -> np.ndarray:
    """[num][4] float32 (pos_u, pos_v, strength, inv_sigma_sq); params laid out as sbs_branched_params."""
    out = np.empty((num, 4), dtype=np.float32)
    lib().orc_branched_scatterers(C.cast(C.byref(params), C.c_void_p), int(num), float(time), _p(out))
    return out


def branched_flow(params, thickness, scatterers, texture, fade: bool) -> np.ndarray:
    """One fade + trace step; returns the updated [tex_height][tex_width] u32 texture."""
    th = np.ascontiguousarray(thickness, dtype=np.float32)
    sc = np.ascontiguousarray(scatterers, dtype=np.float32).reshape(-1, 4)
    tex = np.array(texture, dtype=np.uint32, copy=True)
    lib().orc_branched_flow(C.cast(C.byref(params), C.c_void_p), _p(th), th.shape[1], th.shape[0], th.shape[1],
                            _p(sc), _p(tex), 1 if fade else 0)
    return tex


# ---------------------------------------------------------------------- foam cluster dynamics
def foam_forces(physics, position, radius, velocity=None, thickness_nm=None) -> np.ndarray:
    """compute_forces (foam_dynamics.rs:62-94): [n][3] float32; physics laid out as sbs_foam_physics."""
    pos = np.ascontiguousarray(position, dtype=np.float32).reshape(-1, 3)
    n = pos.shape[0]
    r = np.ascontiguousarray(radius, dtype=np.float32).reshape(n)
    v = None if velocity is None else np.ascontiguousarray(velocity, dtype=np.float32).reshape(n, 3)
    t = None if thickness_nm is None else np.ascontiguousarray(thickness_nm, dtype=np.float32).reshape(n)
    out = np.empty((n, 3), dtype=np.float32)
    lib().orc_foam_forces(C.cast(C.byref(physics), C.c_void_p), n, _p(pos), None if v is None else _p(v), _p(r),
                          None if t is None else _p(t), _p(out))
    return out


def foam_forces_subset(physics, position, radius, idx, velocity=None, thickness_nm=None) -> np.ndarray:
    """The forces on the bubbles idx alone, in compute_forces' accumulation order: [len(idx)][3]."""
    pos = np.ascontiguousarray(position, dtype=np.float32).reshape(-1, 3)
    n = pos.shape[0]
    r = np.ascontiguousarray(radius, dtype=np.float32).reshape(n)
    v = None if velocity is None else np.ascontiguousarray(velocity, dtype=np.float32).reshape(n, 3)
    t = None if thickness_nm is None else np.ascontiguousarray(thickness_nm, dtype=np.float32).reshape(n)
    ix = np.ascontiguousarray(idx, dtype=np.uint32)
    out = np.empty((ix.size, 3), dtype=np.float32)
    lib().orc_foam_forces_subset(C.cast(C.byref(physics), C.c_void_p), n, _p(pos), None if v is None else _p(v), _p(r),
                                 None if t is None else _p(t), _p(ix), ix.size, _p(out))
    return out


def pow15(x: float) -> float:
    return float(lib().orc_pow15(float(x)))


def foam_step(physics, dt: float, steps: int, position, radius, velocity=None, thickness_nm=None, ids=None,
              next_id=None):
    """`steps` FoamSimulator::step calls on the cluster (arrays in cluster order). Returns a dict with
    position, velocity [m][3], radius, thickness_nm [m], ids [m], next_id and connections: a structured
    array of (bubble_a, bubble_b, contact_point[3], contact_normal[3], wall_curvature_radius,
    wall_thickness_nm) in the reference's order."""
    pos = np.array(position, dtype=np.float32, copy=True).reshape(-1, 3)
    n = pos.shape[0]
    r = np.array(radius, dtype=np.float32, copy=True).reshape(n)
    v = np.zeros((n, 3), np.float32) if velocity is None else np.array(velocity, np.float32, copy=True).reshape(n, 3)
    t = np.full(n, 500.0, np.float32) if thickness_nm is None else np.array(thickness_nm, np.float32,
                                                                              copy=True).reshape(n)
    i = np.arange(n, dtype=np.uint32) if ids is None else np.array(ids, dtype=np.uint32, copy=True).reshape(n)
    nid = C.c_uint32(n if next_id is None else int(next_id))
    cap = 64 * n + 64
    conn = np.zeros(cap, dtype=FOAM_CONNECTION)
    nconn = C.c_uint32(0)
    m = lib().orc_foam_step(C.cast(C.byref(physics), C.c_void_p), float(dt), int(steps), n, _p(pos), _p(v), _p(r),
                            _p(t), _p(i), C.byref(nid), conn.ctypes.data, cap, C.byref(nconn))
    if nconn.value > cap:
        raise RuntimeError("connection buffer too small")
    return dict(position=pos[:m], velocity=v[:m], radius=r[:m], thickness_nm=t[:m], ids=i[:m], next_id=nid.value,
                connections=conn[:nconn.value].copy())


FOAM_CONNECTION = np.dtype([("bubble_a", np.uint32), ("bubble_b", np.uint32), ("contact_point", np.float32, 3),
                            ("contact_normal", np.float32, 3), ("wall_curvature_radius", np.float32),
                            ("wall_thickness_nm", np.float32)])


def fix_ring_mean(words, np_):
    """The kernels' exact pole-ring mean of f32 words over a ring of np_ cells."""
    a = np.ascontiguousarray(words, dtype=np.float32).reshape(-1)
    return lib().orc_fix_ring_mean(_p(a), a.size, int(np_))
