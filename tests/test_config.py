"""config.rs:426-465 unit tests on the Python mirror of SimulationConfig (host only)."""
import json

from soap_bubble_simulation_gb300 import SimulationConfig

EPS = 2.220446049250313e-16


def test_default_config():
    c = SimulationConfig.default()
    assert abs(c.bubble.diameter - 0.05) < EPS
    assert abs(c.bubble.film_thickness_nm - 500.0) < EPS
    assert abs(c.fluid.viscosity - 0.001) < EPS
    assert abs(c.environment.gravity - 9.81) < EPS
    assert c.dt == 0.001 and c.resolution == 128


def test_bubble_radius():
    assert abs(SimulationConfig.default().bubble_radius() - 0.025) < EPS


def test_internal_pressure():
    assert abs(SimulationConfig.default().internal_pressure_difference() - 4.0) < 1e-10


def test_film_thickness_conversion():
    assert abs(SimulationConfig.default().film_thickness_meters() - 500e-9) < EPS


def test_serialization_roundtrip(tmp_path):
    c = SimulationConfig.default()
    p = tmp_path / "c.json"
    c.to_file(p)
    d = SimulationConfig.from_file(p)
    assert abs(c.bubble.diameter - d.bubble.diameter) < EPS
    assert d == c


def test_reference_json_layout(tmp_path):
    """The reference's config/default.json layout (no wind/buoyancy/foam keys) parses."""
    text = {
        "bubble": {"diameter": 0.05, "film_thickness_nm": 500.0, "critical_thickness_nm": 10.0,
                   "refractive_index": 1.33},
        "fluid": {"viscosity": 0.001, "surface_tension": 0.025, "density": 1000.0, "surfactant_diffusion": 1e-9,
                  "surfactant_concentration": 0.5},
        "environment": {"gravity": 9.81, "temperature": 293.15, "pressure": 101325.0},
        "dt": 0.001,
        "resolution": 128,
    }
    p = tmp_path / "d.json"
    p.write_text(json.dumps(text))
    c = SimulationConfig.from_file(p)
    assert c == SimulationConfig.default()


def test_to_c_struct():
    c = SimulationConfig.default().to_c()
    assert c.resolution == 128 and c.diameter == 0.05 and c.surfactant_diffusion == 1e-9
