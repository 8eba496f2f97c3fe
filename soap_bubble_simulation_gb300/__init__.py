"""GB300-native film-drainage and thin-film-interference path of the soap-bubble simulation.

Drop-in for the reference's `physics::drainage`, `physics::interference` and
`render::{gpu_drainage, interference_lut}` APIs, plus the bubble fragment shader as a headless
frame (`render_frame`), computed by hand-written
CUDA kernels for sm_103a behind the C ABI in include/sbs.h (libsbs.so).
"""
from . import _native
from .config import (BubbleParameters, ConfigError, EnvironmentParameters, FluidParameters,
                     SimulationConfig)
from .drainage import (DeviceField, DrainageParams, DrainageSimulator, GPUDrainageSimulator,
                       ThicknessField, film_volume_device)
from .interference import (LUT_ANGLE_SAMPLES, LUT_MAX_THICKNESS_NM, LUT_THICKNESS_SAMPLES,
                           FresnelCoefficients, InterferenceCalculator, RgbColor, constants,
                           generate_interference_lut, generate_interference_lut_array, lookup_2d,
                           sample_interference_lut, schlick_interference_rgb, spectral_rgb, wavelengths)
from ._native import SbsError
from .foam import FoamDrainage
from .surrogate import SURROGATE_STEPS, DrainageSurrogate, field_params, masked_error
from .shading import BubbleUniform, Camera, render_frame, shade_fragments
from .caustics import CausticParams, caustic_map
from .branched import BranchedFlowParams, BranchedFlowSimulator, branched_flow_step, generate_scatterers
from .foam_dynamics import FoamPhysics, FoamSimulator, SpatialHash, default_cluster, fcc_foam

__all__ = [
    "BubbleParameters", "ConfigError", "EnvironmentParameters", "FluidParameters", "SimulationConfig",
    "DeviceField", "DrainageParams", "DrainageSimulator", "GPUDrainageSimulator", "ThicknessField",
    "film_volume_device", "LUT_ANGLE_SAMPLES", "LUT_MAX_THICKNESS_NM", "LUT_THICKNESS_SAMPLES",
    "FresnelCoefficients", "InterferenceCalculator", "RgbColor", "constants", "generate_interference_lut",
    "generate_interference_lut_array", "lookup_2d", "sample_interference_lut", "schlick_interference_rgb", "spectral_rgb",
    "wavelengths", "SbsError", "FoamDrainage", "SURROGATE_STEPS", "DrainageSurrogate", "field_params",
    "masked_error", "BubbleUniform", "Camera", "render_frame", "shade_fragments", "CausticParams", "caustic_map",
    "BranchedFlowParams", "BranchedFlowSimulator", "branched_flow_step", "generate_scatterers", "FoamPhysics",
    "FoamSimulator", "SpatialHash", "default_cluster", "fcc_foam",
]
