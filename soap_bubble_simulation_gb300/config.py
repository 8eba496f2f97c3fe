"""SimulationConfig and its parameter groups (config.rs:10-424).

Same field names, defaults and JSON layout as the reference, so a config file
written for the reference loads here unchanged. `to_c()` packs the values the
drainage solver uses into the C struct `sbs_config`.
"""
from __future__ import annotations

import json
from dataclasses import asdict, dataclass, field
from typing import Any

from . import _native as N


class ConfigError(Exception):
    """ConfigError (config.rs:375-424): I/O, parse or serialise failure."""


@dataclass
class BubbleParameters:
    """config.rs:12-35."""

    diameter: float = 0.05
    film_thickness_nm: float = 500.0
    critical_thickness_nm: float = 10.0
    refractive_index: float = 1.33


@dataclass
class FluidParameters:
    """config.rs:38-66."""

    viscosity: float = 0.001
    surface_tension: float = 0.025
    density: float = 1000.0
    surfactant_diffusion: float = 1e-9
    surfactant_concentration: float = 0.5


@dataclass
class EnvironmentParameters:
    """config.rs:70-103 (wind and buoyancy have serde defaults)."""

    gravity: float = 9.81
    temperature: float = 293.15
    pressure: float = 101325.0
    wind: list = field(default_factory=lambda: [0.0, 0.0, 0.0])
    buoyancy: float = 1.0


@dataclass
class SimulationConfig:
    """SimulationConfig (config.rs:283-302) with Default (config.rs:305-316).

    `foam` is carried through as a plain dict: the foam subsystem is not part
    of the physics path this library accelerates.
    """

    bubble: BubbleParameters = field(default_factory=BubbleParameters)
    fluid: FluidParameters = field(default_factory=FluidParameters)
    environment: EnvironmentParameters = field(default_factory=EnvironmentParameters)
    foam: dict = field(default_factory=dict)
    dt: float = 0.001
    resolution: int = 128

    @classmethod
    def default(cls) -> "SimulationConfig":
        return cls()

    @classmethod
    def from_dict(cls, d: dict[str, Any]) -> "SimulationConfig":
        try:
            env = dict(d["environment"])
            return cls(
                bubble=BubbleParameters(**d["bubble"]),
                fluid=FluidParameters(**d["fluid"]),
                environment=EnvironmentParameters(**env),
                foam=dict(d.get("foam", {})),
                dt=float(d["dt"]),
                resolution=int(d["resolution"]),
            )
        except (KeyError, TypeError, ValueError) as e:
            raise ConfigError(f"parse error: {e}") from e

    @classmethod
    def from_file(cls, path) -> "SimulationConfig":
        """SimulationConfig::from_file (config.rs:328-337)."""
        try:
            with open(path) as f:
                text = f.read()
        except OSError as e:
            raise ConfigError(f"io error reading {path}: {e}") from e
        try:
            d = json.loads(text)
        except json.JSONDecodeError as e:
            raise ConfigError(f"parse error in {path}: {e}") from e
        return cls.from_dict(d)

    def to_dict(self) -> dict[str, Any]:
        d = asdict(self)
        if not d["foam"]:
            d.pop("foam")
        return d

    def to_file(self, path) -> None:
        """SimulationConfig::to_file (config.rs:347-354)."""
        try:
            with open(path, "w") as f:
                json.dump(self.to_dict(), f, indent=2)
        except OSError as e:
            raise ConfigError(f"io error writing {path}: {e}") from e

    def bubble_radius(self) -> float:
        """config.rs:357-359."""
        return self.bubble.diameter / 2.0

    def internal_pressure_difference(self) -> float:
        """Young-Laplace, 4 gamma / R (config.rs:363-365)."""
        return 4.0 * self.fluid.surface_tension / self.bubble_radius()

    def film_thickness_meters(self) -> float:
        """config.rs:368-370."""
        return self.bubble.film_thickness_nm * 1e-9

    def to_c(self) -> N.SbsConfig:
        c = N.SbsConfig()
        c.diameter = self.bubble.diameter
        c.film_thickness_nm = self.bubble.film_thickness_nm
        c.critical_thickness_nm = self.bubble.critical_thickness_nm
        c.refractive_index = self.bubble.refractive_index
        c.viscosity = self.fluid.viscosity
        c.surface_tension = self.fluid.surface_tension
        c.density = self.fluid.density
        c.surfactant_diffusion = self.fluid.surfactant_diffusion
        c.surfactant_concentration = self.fluid.surfactant_concentration
        c.gravity = self.environment.gravity
        c.temperature = self.environment.temperature
        c.pressure = self.environment.pressure
        c.dt = self.dt
        c.resolution = int(self.resolution)
        return c
