"""Thin-film interference colour, backed by the CUDA kernels of libsbs.

Mirrors `InterferenceCalculator` (interference.rs:127-512), `RgbColor`
(:41-95), `FresnelCoefficients` (:97-106), the wavelength and index constants
(:24-39), `generate_interference_lut` (interference_lut.rs:18-41), the
Schlick / transmitted-Airy evaluation of wall.wgsl:176-207 and the LUT
lookup of bubble.wgsl:425-439. Scalar methods evaluate a batch of one point
on the GPU; the *_batch methods take numpy arrays.
"""
from __future__ import annotations

import ctypes as C
import math
from dataclasses import dataclass

import numpy as np

from . import _native as N


class wavelengths:  # noqa: N801 - module-like namespace as in the reference
    """interference.rs:24-31."""

    RED_NM = 650.0
    GREEN_NM = 532.0
    BLUE_NM = 450.0


class constants:  # noqa: N801
    """interference.rs:34-39."""

    REFRACTIVE_INDEX_AIR = 1.0
    REFRACTIVE_INDEX_SOAP_FILM = 1.33


LUT_THICKNESS_SAMPLES = 256
LUT_ANGLE_SAMPLES = 64
LUT_MAX_THICKNESS_NM = 2000.0


def _clamp01(x: float) -> float:
    if x != x:  # NaN passes through f64::clamp
        return x
    return min(max(x, 0.0), 1.0)


def _round_half_away(x: float) -> int:
    return int(math.floor(x + 0.5)) if x >= 0 else -int(math.floor(-x + 0.5))


@dataclass
class RgbColor:
    """RGB colour in [0, 1] (interference.rs:41-95)."""

    red: float = 0.0
    green: float = 0.0
    blue: float = 0.0

    @classmethod
    def new(cls, red: float, green: float, blue: float) -> "RgbColor":
        return cls(_clamp01(red), _clamp01(green), _clamp01(blue))

    @classmethod
    def from_f32(cls, red: float, green: float, blue: float) -> "RgbColor":
        f = np.float32
        return cls.new(float(f(red)), float(f(green)), float(f(blue)))

    @classmethod
    def default(cls) -> "RgbColor":
        return cls()

    def to_f32_tuple(self) -> tuple[float, float, float]:
        f = np.float32
        return (float(f(self.red)), float(f(self.green)), float(f(self.blue)))

    def to_u8_tuple(self) -> tuple[int, int, int]:
        """(x * 255).round() as u8: round half away from zero, saturating."""
        return tuple(max(0, min(255, _round_half_away(c * 255.0))) for c in (self.red, self.green, self.blue))

    def to_f32_array_with_alpha(self, alpha: float) -> list[float]:
        return [*self.to_f32_tuple(), float(np.float32(alpha))]


@dataclass
class FresnelCoefficients:
    """interference.rs:97-106."""

    reflectance_s: float
    reflectance_p: float
    reflectance_average: float


def _arr(x, dtype=np.float64) -> np.ndarray:
    return np.ascontiguousarray(np.asarray(x, dtype=dtype).reshape(-1))


def _terms(n: float, wl: float, t, ci) -> np.ndarray:
    t = _arr(t)
    ci = _arr(ci)
    out = np.empty((t.size, 8), dtype=np.float64)
    N.call("sbs_interference_terms_batch", float(n), float(wl), N.ptr(t), N.ptr(ci), t.size, N.ptr(out), N.MEM_HOST,
           None)
    return out


class InterferenceCalculator:
    """InterferenceCalculator (interference.rs:127-512): three-wavelength two-beam/Airy colour."""

    def __init__(self, refractive_index_film: float = constants.REFRACTIVE_INDEX_SOAP_FILM):
        self._n = float(refractive_index_film)
        self._n_medium = constants.REFRACTIVE_INDEX_AIR
        self._wl = np.array([wavelengths.RED_NM, wavelengths.GREEN_NM, wavelengths.BLUE_NM], dtype=np.float64)

    @classmethod
    def new(cls, refractive_index_film: float) -> "InterferenceCalculator":
        return cls(refractive_index_film)

    @classmethod
    def default_soap_film(cls) -> "InterferenceCalculator":
        return cls(constants.REFRACTIVE_INDEX_SOAP_FILM)

    @classmethod
    def default(cls) -> "InterferenceCalculator":
        return cls.default_soap_film()

    @classmethod
    def with_custom_wavelengths(cls, refractive_index_film: float, red_nm: float, green_nm: float,
                                blue_nm: float) -> "InterferenceCalculator":
        c = cls(refractive_index_film)
        c._wl = np.array([red_nm, green_nm, blue_nm], dtype=np.float64)
        return c

    def refractive_index_film(self) -> float:
        return self._n

    def refractive_index_medium(self) -> float:
        return self._n_medium

    def wavelengths_nm(self) -> tuple[float, float, float]:
        return tuple(float(w) for w in self._wl)

    # --- scalar terms (interference.rs:197-353), each a one-point GPU batch ---------------
    def calculate_transmission_angle_cos(self, cos_theta_incident: float) -> float:
        return float(_terms(self._n, 550.0, [1.0], [cos_theta_incident])[0, 0])

    def calculate_optical_path_difference(self, film_thickness_nm: float, cos_theta_transmitted: float,
                                          wavelength_nm: float) -> float:
        return float(self.optical_path_difference_batch([film_thickness_nm], [cos_theta_transmitted],
                                                        [wavelength_nm])[0])

    def calculate_phase_difference(self, optical_path_difference_nm: float, wavelength_nm: float) -> float:
        return float(self.phase_difference_batch([optical_path_difference_nm], [wavelength_nm])[0])

    def calculate_fresnel_reflection(self, cos_theta_incident: float) -> FresnelCoefficients:
        o = _terms(self._n, 550.0, [1.0], [cos_theta_incident])[0]
        return FresnelCoefficients(float(o[3]), float(o[4]), float(o[5]))

    def calculate_reflected_intensity(self, film_thickness_nm: float, cos_theta_incident: float,
                                      wavelength_nm: float) -> float:
        return float(_terms(self._n, wavelength_nm, [film_thickness_nm], [cos_theta_incident])[0, 6])

    def calculate_interference_color(self, film_thickness_nm: float, cos_theta_incident: float) -> RgbColor:
        c = self.color_batch([film_thickness_nm], [cos_theta_incident], gamma=True)[0]
        return RgbColor(float(c[0]), float(c[1]), float(c[2]))

    def calculate_interference_color_linear(self, film_thickness_nm: float, cos_theta_incident: float) -> RgbColor:
        c = self.color_batch([film_thickness_nm], [cos_theta_incident], gamma=False)[0]
        return RgbColor(float(c[0]), float(c[1]), float(c[2]))

    def calculate_interference_color_with_index(self, film_thickness_nm: float, cos_theta_incident: float,
                                                refractive_index: float) -> RgbColor:
        return InterferenceCalculator(refractive_index).calculate_interference_color(film_thickness_nm,
                                                                                     cos_theta_incident)

    # --- batches --------------------------------------------------------------------------
    def color_batch(self, film_thickness_nm, cos_theta_incident, gamma: bool = True,
                    precision: str = "f64") -> np.ndarray:
        """Colours for arrays of thickness (nm) and cos(theta): [n, 3]. precision 'f64' or 'f32'."""
        dt = np.float64 if precision == "f64" else np.float32
        prec = N.PREC_F64 if precision == "f64" else N.PREC_F32
        t = _arr(film_thickness_nm, dt)
        ci = _arr(cos_theta_incident, dt)
        if t.size != ci.size:
            raise ValueError("thickness and cos arrays differ in length")
        out = np.empty((t.size, 3), dtype=dt)
        N.call("sbs_interference_color_batch", self._n, N.dptr(self._wl), N.ptr(t), N.ptr(ci), t.size,
               1 if gamma else 0, prec, N.ptr(out), N.MEM_HOST, None)
        return out

    def terms_batch(self, film_thickness_nm, cos_theta_incident, wavelength_nm: float) -> np.ndarray:
        """[n, 8]: cos_t, opd, phase, Rs, Rp, R, intensity, 0."""
        return _terms(self._n, wavelength_nm, film_thickness_nm, cos_theta_incident)

    def optical_path_difference_batch(self, t_nm, cos_t, wl_nm) -> np.ndarray:
        t, c, w = _arr(t_nm), _arr(cos_t), _arr(wl_nm)
        out = np.empty_like(t)
        N.call("sbs_optical_path_batch", self._n, N.ptr(t), N.ptr(c), N.ptr(w), t.size, N.ptr(out), N.MEM_HOST, None)
        return out

    def phase_difference_batch(self, opd_nm, wl_nm) -> np.ndarray:
        o, w = _arr(opd_nm), _arr(wl_nm)
        out = np.empty_like(o)
        N.call("sbs_phase_difference_batch", N.ptr(o), N.ptr(w), o.size, N.ptr(out), N.MEM_HOST, None)
        return out

    # --- lookup tables ---------------------------------------------------------------------
    def color_lookup_array(self, min_thickness_nm: float, max_thickness_nm: float, num_samples: int,
                           cos_theta: float) -> np.ndarray:
        out = np.empty((num_samples, 3), dtype=np.float64)
        N.call("sbs_lut1d_build", self._n, N.dptr(self._wl), float(min_thickness_nm), float(max_thickness_nm),
               int(num_samples), float(cos_theta), N.ptr(out), N.MEM_HOST, None)
        return out

    def generate_color_lookup_table(self, min_thickness_nm: float, max_thickness_nm: float, num_samples: int,
                                    cos_theta: float) -> list[RgbColor]:
        """interference.rs:461-477."""
        a = self.color_lookup_array(min_thickness_nm, max_thickness_nm, num_samples, cos_theta)
        return [RgbColor(*map(float, row)) for row in a]

    def color_lookup_2d_array(self, min_thickness_nm: float, max_thickness_nm: float, thickness_samples: int,
                              angle_samples: int) -> np.ndarray:
        """[thickness][angle][3] f64 table."""
        out = np.empty((thickness_samples, angle_samples, 3), dtype=np.float64)
        N.call("sbs_lut2d_build", self._n, N.dptr(self._wl), float(min_thickness_nm), float(max_thickness_nm),
               int(thickness_samples), int(angle_samples), N.ptr(out), N.MEM_HOST, None)
        return out

    def generate_2d_color_lookup_table(self, min_thickness_nm: float, max_thickness_nm: float,
                                       thickness_samples: int, angle_samples: int) -> list[list[RgbColor]]:
        """interference.rs:491-512."""
        a = self.color_lookup_2d_array(min_thickness_nm, max_thickness_nm, thickness_samples, angle_samples)
        return [[RgbColor(*map(float, c)) for c in row] for row in a]


def generate_interference_lut(refractive_index: float, intensity: float) -> bytes:
    """RGBA8 LUT [64 angle][256 thickness][4] over 0-2000 nm (interference_lut.rs:18-41)."""
    out = np.empty(LUT_THICKNESS_SAMPLES * LUT_ANGLE_SAMPLES * 4, dtype=np.uint8)
    N.call("sbs_interference_lut_rgba8", float(refractive_index), float(intensity), N.ptr(out), N.MEM_HOST, None)
    return out.tobytes()


def generate_interference_lut_array(refractive_index: float, intensity: float) -> np.ndarray:
    return np.frombuffer(generate_interference_lut(refractive_index, intensity), dtype=np.uint8).reshape(
        LUT_ANGLE_SAMPLES, LUT_THICKNESS_SAMPLES, 4)


def schlick_interference_rgb(film_thickness_nm, cos_theta_incident, refractive_index: float,
                             wavelengths_nm=(650.0, 532.0, 450.0)) -> np.ndarray:
    """wall.wgsl:176-207: Schlick reflectance with the transmitted Airy term, [n, 3] f32."""
    t = _arr(film_thickness_nm, np.float32)
    ci = _arr(cos_theta_incident, np.float32)
    wl = np.asarray(wavelengths_nm, dtype=np.float32)
    out = np.empty((t.size, 3), dtype=np.float32)
    N.call("sbs_schlick_rgb_batch", float(refractive_index), wl.ctypes.data_as(C.POINTER(C.c_float)), N.ptr(t),
           N.ptr(ci), t.size, N.ptr(out), N.MEM_HOST, None)
    return out


def sample_interference_lut(lut: np.ndarray, film_thickness_nm, cos_theta, intensity: float = 1.0,
                            max_thickness_nm: float = LUT_MAX_THICKNESS_NM, addressing: str = "texel") -> np.ndarray:
    """bubble.wgsl:425-439 lookup of an RGBA8 LUT [H][W][4]; addressing 'texel' (the sampler of
    pipeline.rs:350-359) or 'grid'. Returns [n, 3] f32."""
    L = np.ascontiguousarray(lut, dtype=np.uint8)
    H, W = L.shape[0], L.shape[1]
    t = _arr(film_thickness_nm, np.float32)
    ci = _arr(cos_theta, np.float32)
    out = np.empty((t.size, 3), dtype=np.float32)
    mode = N.LOOKUP_TEXEL if addressing == "texel" else N.LOOKUP_GRID
    N.call("sbs_lut_rgba8_lookup_batch", N.ptr(L), W, H, float(max_thickness_nm), float(intensity), mode, N.ptr(t),
           N.ptr(ci), t.size, N.ptr(out), N.MEM_HOST, None)
    return out


def lookup_2d(lut: np.ndarray, tmin: float, tmax: float, film_thickness_nm, cos_theta) -> np.ndarray:
    """Grid-aligned bilinear read of a [T][A][3] f64 LUT. Returns [n, 3] f64."""
    L = np.ascontiguousarray(lut, dtype=np.float64)
    t = _arr(film_thickness_nm)
    ci = _arr(cos_theta)
    out = np.empty((t.size, 3), dtype=np.float64)
    N.call("sbs_lut2d_lookup_batch", N.ptr(L), L.shape[0], L.shape[1], float(tmin), float(tmax), N.ptr(t), N.ptr(ci),
           t.size, N.ptr(out), N.MEM_HOST, None)
    return out


def spectral_rgb(film_thickness_nm, cos_theta, refractive_index, wavelengths_nm, cmf, mode: str = "tc") -> np.ndarray:
    """Per point: Airy reflectance at each wavelength contracted with the [nl, 3] colour-matching
    matrix. mode 'tc' = BF16 tensor-core contraction (tcgen05, FP32 accumulation), 'fp32' = FP32
    throughout. Returns [n, 3] f32."""
    t = _arr(film_thickness_nm, np.float32)
    ci = _arr(cos_theta, np.float32)
    nf = _arr(refractive_index, np.float32)
    wl = _arr(wavelengths_nm, np.float32)
    m = np.ascontiguousarray(np.asarray(cmf, dtype=np.float32).reshape(-1, 3))
    if m.shape[0] != wl.size:
        raise ValueError("cmf must have one row per wavelength")
    out = np.empty((t.size, 3), dtype=np.float32)
    md = N.SPECTRAL_TC_BF16 if mode == "tc" else N.SPECTRAL_FP32
    N.call("sbs_spectral_rgb", N.ptr(t), N.ptr(ci), N.ptr(nf), t.size, N.ptr(wl), wl.size, N.ptr(m), md, N.ptr(out),
           N.MEM_HOST, None)
    return out
