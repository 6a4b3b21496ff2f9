"""Host-side configuration: the reference's YAML schema, validation and the
block layout rule (src/mesh.rs:358-397)."""
import math

import pytest

from knc import config, setups, workloads

SETUP = """
hydro:
  relativistic:
    gamma_law_index: 1.3333333333333333
    plm_theta: 1.5
    cfl_number: 0.4
    runge_kutta_order: RK2
    riemann_solver: HLLE   # HLLC also accepted

model:
  wind:
    rho0: 1.0
    ur: 1.0
    temperature: 1.e-4
    noise: 0.01

mesh:
  reference_radius: 1.0
  inner_radius: 1.0
  outer_radius: 10.0
  inner_excision_speed: 0.0
  outer_excision_speed: 0.0
  num_polar_zones: 128
  num_radial_zones: 82
  block_size: 64

control:
  start_time: 0.0
  final_time: 1e-10
  checkpoint_interval: 1e-11
  fold: 10
  num_threads: ~
  output_directory: data
"""


def test_parse_setup():
    c = setups.load_setup(SETUP)
    assert isinstance(c.hydro, config.RelativisticHydro)
    assert c.hydro.riemann_solver == "HLLE" and c.hydro.adaptive_time_step is False
    assert c.mesh.num_radial_zones == 82 and c.mesh.excision_delay is None
    assert c.control.num_threads is None and c.control.fold == 10
    assert c.device_model().temperature == 1e-4
    assert c.mesh.grid_block_indexes() == [0, 1, 2, 3]


def test_unknown_field_rejected():
    with pytest.raises(config.ConfigError, match="unknown field"):
        setups.load_setup(SETUP.replace("cfl_number: 0.4", "cfl_number: 0.4\n    eta_0: 1.0"))


@pytest.mark.parametrize("edit,msg", [
    ("plm_theta: 1.5", "plm_theta"),
    ("cfl_number: 0.4", "cfl_number"),
])
def test_hydro_validation(edit, msg):
    bad = SETUP.replace(edit, edit.split(":")[0] + ": 3.0")
    with pytest.raises(config.ConfigError, match=msg):
        setups.load_setup(bad)


def test_mesh_validation():
    with pytest.raises(config.ConfigError, match="inner_excision_speed"):
        setups.load_setup(SETUP.replace("inner_excision_speed: 0.0", "inner_excision_speed: 5.0"))
    with pytest.raises(config.ConfigError, match="16 polar"):
        setups.load_setup(SETUP.replace("num_polar_zones: 128", "num_polar_zones: 8"))


def test_yaml_scalars():
    d = setups.parse_yaml("a:\n  b: 1e-3\n  c: 1.e9\n  d: 50e9\n  e: ~\n  f: true\n  g: 'x # y'\n  h: 4\n")
    assert d["a"] == {"b": 1e-3, "c": 1e9, "d": 50e9, "e": None, "f": True, "g": "x # y", "h": 4}


def test_block_layouts():
    assert workloads.wind_small().num_blocks == 4
    assert workloads.wind_large().num_blocks == 64
    assert workloads.jet().num_blocks == 32
    r0, r1 = workloads.wind_large().mesh.block_radii(63)
    assert r1 == pytest.approx(10.0008, abs=2e-4)
    m = workloads.wind_small().mesh
    assert m.block_radii(1)[0] == pytest.approx((1 + 64 / 82) ** 1)
    assert math.isclose(m.zone_dlogr(), 1 / 82)
