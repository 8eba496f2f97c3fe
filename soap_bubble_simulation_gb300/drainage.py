"""Film drainage on the bubble's theta-phi grid, backed by the CUDA kernels of libsbs.

Mirrors the reference's two solvers with their method names:

* `DrainageSimulator` (drainage.rs:212-614): CPU semantics, forward Euler of
  dh/dt = -rho g h^3/(3 eta) sin(theta) + D lap(h), pole rings averaged each
  step, marginal-regeneration (TFE) fronts.
* `GPUDrainageSimulator` (gpu_drainage.rs:81-490): WGSL semantics, the same
  stencil co-evolving a surfactant field with optional Marangoni coupling,
  pole rows held fixed.

Both keep their fields in GPU memory as f32; every step, query and reduction
runs on the GPU. `ThicknessField` is the host container of the reference
(drainage.rs:96-204), used for snapshots and for building initial fields.
"""
from __future__ import annotations

import ctypes as C
import math
from dataclasses import dataclass, fields

import numpy as np

from . import _native as N
from .config import SimulationConfig


class ThicknessField:
    """Row-major [theta][phi] thickness grid in metres (drainage.rs:96-204), host side."""

    def __init__(self, num_theta: int, num_phi: int, initial_thickness: float):
        self._nt = int(num_theta)
        self._np = int(num_phi)
        self._data = np.full(self._nt * self._np, float(initial_thickness), dtype=np.float64)
        self._dth = math.pi / (self._nt - 1)
        self._dph = 2.0 * math.pi / self._np

    @classmethod
    def from_array(cls, a: np.ndarray) -> "ThicknessField":
        a = np.asarray(a, dtype=np.float64)
        f = cls(a.shape[0], a.shape[1], 0.0)
        f._data[:] = a.reshape(-1)
        return f

    def get(self, theta_index: int, phi_index: int) -> float:
        return float(self._data[theta_index * self._np + phi_index])

    def set(self, theta_index: int, phi_index: int, value: float) -> None:
        self._data[theta_index * self._np + phi_index] = value

    def theta_at(self, theta_index: int) -> float:
        return theta_index * self._dth

    def phi_at(self, phi_index: int) -> float:
        return phi_index * self._dph

    def num_theta(self) -> int:
        return self._nt

    def num_phi(self) -> int:
        return self._np

    def delta_theta(self) -> float:
        return self._dth

    def delta_phi(self) -> float:
        return self._dph

    def min_thickness(self) -> float:
        return float(self._data.min())

    def max_thickness(self) -> float:
        return float(self._data.max())

    def data(self) -> np.ndarray:
        """Read-only view of the flat data."""
        v = self._data.view()
        v.flags.writeable = False
        return v

    def data_mut(self) -> np.ndarray:
        return self._data

    def as_array(self) -> np.ndarray:
        return self._data.reshape(self._nt, self._np)


@dataclass
class DeviceField:
    """A device-resident f32 field: `ptr` is a device address, rows are `pitch` elements apart.

    Stands in for the `&wgpu::Buffer` the reference's getters return; valid until the next step,
    run or set call on the simulator that produced it.
    """

    ptr: int
    pitch: int
    num_theta: int
    num_phi: int
    stream: int

    def nbytes(self) -> int:
        return self.pitch * self.num_theta * 4


class _Handle:
    """Owns one sbs_drainage handle."""

    def __init__(self):
        self._h = C.c_void_p()

    @property
    def handle(self) -> C.c_void_p:
        if not self._h:
            raise N.SbsError(N.SBS_E_STATE, "simulator is closed")
        return self._h

    def close(self) -> None:
        if self._h:
            N.lib().sbs_drainage_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    # shared helpers -----------------------------------------------------------------
    def grid(self) -> tuple[int, int]:
        nt, np_ = C.c_uint32(), C.c_uint32()
        N.call("sbs_drainage_grid_size", self.handle, C.byref(nt), C.byref(np_))
        return nt.value, np_.value

    def _field_out(self, fn: str) -> np.ndarray:
        nt, np_ = self.grid()
        out = np.empty((nt, np_), dtype=np.float32)
        N.call(fn, self.handle, N.ptr(out), out.size, N.MEM_HOST)
        return out

    def _field_in(self, fn: str, a) -> None:
        nt, np_ = self.grid()
        a = np.ascontiguousarray(a, dtype=np.float32)
        if a.size != nt * np_:
            raise ValueError(f"field must have {nt} x {np_} values, got {a.shape}")
        N.call(fn, self.handle, N.ptr(a), a.size, N.MEM_HOST)

    def thickness_array(self) -> np.ndarray:
        """Current thickness field as an f32 [theta][phi] array (device to host copy)."""
        return self._field_out("sbs_drainage_get_thickness_field")

    def set_thickness_array(self, a) -> None:
        """Loads a [theta][phi] thickness field (metres)."""
        self._field_in("sbs_drainage_set_thickness", a)

    def set_thickness_device(self, ptr: int, n: int) -> None:
        """Loads a thickness field from a dense device array of n f32 values."""
        N.call("sbs_drainage_set_thickness", self.handle, C.c_void_p(ptr), n, N.MEM_DEVICE)

    def get_thickness_device(self, ptr: int, n: int) -> None:
        """Copies the thickness field into a dense device array of n f32 values."""
        N.call("sbs_drainage_get_thickness_field", self.handle, C.c_void_p(ptr), n, N.MEM_DEVICE)

    def get_thickness(self, theta: float, phi: float) -> float:
        """Bilinear thickness query (drainage.rs:516-552), evaluated on the GPU."""
        out = C.c_double()
        N.call("sbs_drainage_get_thickness", self.handle, float(theta), float(phi), C.byref(out))
        return out.value

    def get_thickness_batch(self, theta, phi) -> np.ndarray:
        t = np.ascontiguousarray(theta, dtype=np.float64).reshape(-1)
        p = np.ascontiguousarray(phi, dtype=np.float64).reshape(-1)
        if t.size != p.size:
            raise ValueError("theta and phi differ in length")
        out = np.empty_like(t)
        N.call("sbs_drainage_query_batch", self.handle, N.ptr(t), N.ptr(p), N.ptr(out), t.size, N.MEM_HOST)
        return out

    def current_time(self) -> float:
        out = C.c_double()
        N.call("sbs_drainage_current_time", self.handle, C.byref(out))
        return out.value

    def min_max(self) -> tuple[float, float]:
        a, b = C.c_double(), C.c_double()
        N.call("sbs_drainage_min_max", self.handle, C.byref(a), C.byref(b))
        return a.value, b.value

    def film_volume(self) -> float:
        """FP64 film volume sum h R^2 sin(theta) dtheta dphi of the current field (m^3)."""
        out = C.c_double()
        N.call("sbs_drainage_film_volume", self.handle, C.byref(out))
        return out.value

    def run_checked(self, dt: float, n: int, check_every: int) -> np.ndarray:
        """Advances n steps with an FP64 volume check after every check_every-th step."""
        k = n // check_every if check_every else 0
        vols = np.zeros(max(k, 1), dtype=np.float64)
        N.call("sbs_drainage_run_checked", self.handle, float(dt), int(n), int(check_every), N.dptr(vols))
        return vols[:k]

    def stream(self) -> int:
        out = C.c_void_p()
        N.call("sbs_drainage_stream", self.handle, C.byref(out))
        return out.value or 0

    def vertex_colors(self, xyz, lut, tmin: float, tmax: float) -> np.ndarray:
        """Colours unit vertices from the current field through a [T][A][3] f64 LUT (one kernel)."""
        x = np.ascontiguousarray(xyz, dtype=np.float64).reshape(-1, 3)
        L = np.ascontiguousarray(lut, dtype=np.float64)
        T, A = L.shape[0], L.shape[1]
        out = np.empty_like(x)
        N.call("sbs_drainage_vertex_colors", self.handle, N.ptr(x), x.shape[0], N.ptr(L), T, A, float(tmin),
               float(tmax), N.ptr(out), N.MEM_HOST)
        return out

    def _device_view(self, fn: str, which: int) -> DeviceField:
        p, pitch = C.c_void_p(), C.c_size_t()
        N.call(fn, self.handle, which, C.byref(p), C.byref(pitch))
        nt, np_ = self.grid()
        return DeviceField(p.value or 0, pitch.value, nt, np_, self.stream())


class DrainageSimulator(_Handle):
    """DrainageSimulator (drainage.rs:212-614) on the GPU: CPU semantics in f32.

    Same constructor and methods as the reference. The field lives on the GPU;
    `thickness_field()` returns a host snapshot.
    """

    def __init__(self, config: SimulationConfig | None = None):
        super().__init__()
        self._config = config if config is not None else SimulationConfig.default()
        c = self._config.to_c()
        N.call("sbs_drainage_create", C.byref(c), C.byref(self._h))

    def step(self, dt: float) -> None:
        """One forward-Euler step (drainage.rs:298-392)."""
        N.call("sbs_drainage_step", self.handle, float(dt))

    def step_n(self, dt: float, n: int) -> None:
        """n steps of size dt, replayed as CUDA graphs."""
        N.call("sbs_drainage_step_n", self.handle, float(dt), int(n))

    def thickness_field(self) -> ThicknessField:
        """Snapshot of the field (drainage.rs:555-557), widened to f64."""
        return ThicknessField.from_array(self.thickness_array())

    def set_thickness_field(self, field) -> None:
        """Loads a field (ThicknessField or [theta][phi] array, metres). No reference counterpart:
        the reference can only start from a uniform field."""
        a = field.as_array() if isinstance(field, ThicknessField) else np.asarray(field)
        self.set_thickness_array(a)

    def has_critical_region(self) -> bool:
        out = C.c_int()
        N.call("sbs_drainage_has_critical_region", self.handle, C.byref(out))
        return bool(out.value)

    def critical_thickness(self) -> float:
        out = C.c_double()
        N.call("sbs_drainage_critical_thickness", self.handle, C.byref(out))
        return out.value

    def reset(self, initial_thickness: float) -> None:
        """drainage.rs:575-583."""
        N.call("sbs_drainage_reset", self.handle, float(initial_thickness))

    def set_marginal_regeneration(self, enabled: bool) -> None:
        N.call("sbs_drainage_set_marginal_regeneration", self.handle, 1 if enabled else 0)

    def marginal_regeneration_enabled(self) -> bool:
        out = C.c_int()
        N.call("sbs_drainage_marginal_regeneration_enabled", self.handle, C.byref(out))
        return bool(out.value)

    def set_tfe_thickness_ratio(self, ratio: float) -> None:
        N.call("sbs_drainage_set_tfe_thickness_ratio", self.handle, float(ratio))

    def tfe_thickness_ratio(self) -> float:
        out = C.c_double()
        N.call("sbs_drainage_tfe_thickness_ratio", self.handle, C.byref(out))
        return out.value

    def active_tfe_count(self) -> int:
        out = C.c_uint32()
        N.call("sbs_drainage_active_tfe_count", self.handle, C.byref(out))
        return out.value

    def thickness_device(self) -> DeviceField:
        return self._device_view("sbs_drainage_thickness_device", 0)


@dataclass
class DrainageParams:
    """DrainageParams (gpu_drainage.rs:12-68): the 64-byte uniform with its defaults."""

    dt: float = 0.001
    gravity: float = 9.81
    viscosity: float = 0.001
    density: float = 1000.0
    diffusion_coeff: float = 1e-9
    bubble_radius: float = 0.025
    critical_thickness: float = 30e-9
    grid_width: int = 128
    grid_height: int = 64
    marangoni_enabled: int = 0
    gamma_air: float = 0.072
    gamma_reduction: float = 0.045
    surfactant_diffusion: float = 1e-9
    marangoni_coeff: float = 0.01
    _padding1: int = 0
    _padding2: int = 0

    @classmethod
    def default(cls) -> "DrainageParams":
        return cls()

    def to_c(self) -> N.SbsDrainageParams:
        c = N.SbsDrainageParams()
        for f in fields(self):
            setattr(c, f.name, getattr(self, f.name))
        return c

    @classmethod
    def from_c(cls, c: N.SbsDrainageParams) -> "DrainageParams":
        return cls(**{f.name: getattr(c, f.name) for f in fields(cls)})


class GPUDrainageSimulator(_Handle):
    """GPUDrainageSimulator (gpu_drainage.rs:81-490): WGSL semantics on sm_103a.

    `device` is accepted for signature compatibility and ignored (one GPU,
    the current CUDA device). `step` records nothing into an encoder: it runs
    the passes and returns when they are done.
    """

    def __init__(self, device=None, initial_thickness: float = 500e-9, grid_width: int = 128,
                 grid_height: int = 64):
        super().__init__()
        N.call("sbs_gpu_drainage_create", float(initial_thickness), int(grid_width), int(grid_height),
               C.byref(self._h))
        self._enabled = False
        self._time_scale = 100.0
        self._steps_per_frame = 10
        self._marangoni = False

    # public fields of the reference struct (gpu_drainage.rs:100-107)
    @property
    def enabled(self) -> bool:
        return self._enabled

    @enabled.setter
    def enabled(self, v: bool) -> None:
        N.call("sbs_gpu_drainage_set_enabled", self.handle, 1 if v else 0)
        self._enabled = bool(v)

    @property
    def time_scale(self) -> float:
        return self._time_scale

    @time_scale.setter
    def time_scale(self, v: float) -> None:
        N.call("sbs_gpu_drainage_set_time_scale", self.handle, float(v))
        self._time_scale = float(v)

    @property
    def steps_per_frame(self) -> int:
        return self._steps_per_frame

    @steps_per_frame.setter
    def steps_per_frame(self, v: int) -> None:
        N.call("sbs_gpu_drainage_set_steps_per_frame", self.handle, int(v))
        self._steps_per_frame = int(v)

    @property
    def marangoni_enabled(self) -> bool:
        return self._marangoni

    def step(self, encoder=None, dt: float | None = None) -> None:
        """gpu_drainage.rs:338-370. Called as step(dt) or step(encoder, dt)."""
        if dt is None:
            dt, encoder = encoder, None
        N.call("sbs_gpu_drainage_step", self.handle, float(dt))

    def run(self, passes: int) -> None:
        """`passes` drainage_step passes with params.dt, regardless of `enabled`."""
        N.call("sbs_gpu_drainage_run", self.handle, int(passes))

    def update_params(self, queue_or_params, params: DrainageParams | None = None) -> None:
        p = params if params is not None else queue_or_params
        c = p.to_c()
        N.call("sbs_gpu_drainage_update_params", self.handle, C.byref(c))
        self._marangoni = bool(p.marangoni_enabled)

    def set_dt(self, *args) -> None:
        N.call("sbs_gpu_drainage_set_dt", self.handle, float(args[-1]))

    def set_physics(self, *args) -> None:
        viscosity, density, gravity, diffusion = args[-4:]
        N.call("sbs_gpu_drainage_set_physics", self.handle, float(viscosity), float(density), float(gravity),
               float(diffusion))

    def set_bubble_radius(self, *args) -> None:
        N.call("sbs_gpu_drainage_set_bubble_radius", self.handle, float(args[-1]))

    def reset(self, *args) -> None:
        """gpu_drainage.rs:418-433: both buffers to the thickness, concentration to 0.5."""
        N.call("sbs_drainage_reset", self.handle, float(args[-1]))

    def set_marangoni_enabled(self, *args) -> None:
        en = bool(args[-1])
        N.call("sbs_gpu_drainage_set_marangoni_enabled", self.handle, 1 if en else 0)
        self._marangoni = en

    def set_marangoni_params(self, *args) -> None:
        gamma_air, gamma_reduction, surfactant_diffusion, marangoni_coeff = args[-4:]
        N.call("sbs_gpu_drainage_set_marangoni_params", self.handle, float(gamma_air), float(gamma_reduction),
               float(surfactant_diffusion), float(marangoni_coeff))

    def params(self) -> DrainageParams:
        c = N.SbsDrainageParams()
        N.call("sbs_gpu_drainage_params", self.handle, C.byref(c))
        return DrainageParams.from_c(c)

    def grid_size(self) -> tuple[int, int]:
        """(width, height) = (phi points, theta points), gpu_drainage.rs:482-484."""
        nt, np_ = self.grid()
        return np_, nt

    def concentration_array(self) -> np.ndarray:
        return self._field_out("sbs_drainage_get_concentration_field")

    def set_concentration_array(self, a) -> None:
        self._field_in("sbs_drainage_set_concentration", a)

    def current_thickness_buffer(self) -> DeviceField:
        """The newest thickness field on the device."""
        return self._device_view("sbs_drainage_thickness_device", 0)

    def current_buffer(self) -> DeviceField:
        """What the reference's current_buffer() hands out (gpu_drainage.rs:473-479): after a
        step that is the last pass's input, one pass behind current_thickness_buffer()."""
        return self._device_view("sbs_drainage_thickness_device", 1)

    def caustic_map(self, params=None, which: int = 0) -> np.ndarray:
        """The caustic compute pass (caustics_compute.wgsl) over this simulator's thickness, on its
        stream without a copy of the field. which = 1 reads the buffer the reference's caustic
        renderer binds (current_buffer())."""
        from .caustics import CausticParams

        nt, np_ = self.grid()
        p = params if params is not None else CausticParams.default(np_, nt)
        out = np.empty((nt, np_), dtype=np.float32)
        N.call("sbs_gpu_drainage_caustics", self.handle, C.cast(C.byref(p), C.c_void_p), int(which), N.ptr(out),
               N.MEM_HOST)
        return out

    def run_caustic_map(self, passes: int, params=None) -> np.ndarray:
        """run(passes) followed by caustic_map(params, which=1), with the map written by the run's
        final blocked launch (the field is not read again)."""
        from .caustics import CausticParams

        nt, np_ = self.grid()
        p = params if params is not None else CausticParams.default(np_, nt)
        out = np.empty((nt, np_), dtype=np.float32)
        N.call("sbs_gpu_drainage_run_caustics", self.handle, int(passes), C.cast(C.byref(p), C.c_void_p), N.ptr(out),
               N.MEM_HOST)
        return out

    def step_caustic_map(self, frame_dt: float, params=None) -> np.ndarray:
        """step(frame_dt) followed by the caustic map of the buffer the renderer binds."""
        from .caustics import CausticParams

        nt, np_ = self.grid()
        p = params if params is not None else CausticParams.default(np_, nt)
        out = np.empty((nt, np_), dtype=np.float32)
        N.call("sbs_gpu_drainage_step_caustics", self.handle, float(frame_dt), C.cast(C.byref(p), C.c_void_p),
               N.ptr(out), N.MEM_HOST)
        return out

    def concentration_buffer(self) -> DeviceField:
        """The reference's concentration_buffer() (gpu_drainage.rs:458-460), same indexing as
        current_buffer()."""
        return self._device_view("sbs_drainage_concentration_device", 1)

    def current_concentration_buffer(self) -> DeviceField:
        return self._device_view("sbs_drainage_concentration_device", 0)


def film_volume_device(ptr: int, num_theta: int, num_phi: int, pitch: int, radius: float, stream: int = 0) -> float:
    """FP64 film volume of a device field (no handle needed)."""
    out = C.c_double()
    N.call("sbs_film_volume_device", C.c_void_p(ptr), int(num_theta), int(num_phi), int(pitch), float(radius),
           C.byref(out), C.c_void_p(stream))
    return out.value
