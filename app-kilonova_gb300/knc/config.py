"""Configuration mirrors of the reference's serde structs.

`RelativisticHydro` / `NewtonianHydro` mirror src/physics/relativistic_hydro.rs:15-36
and src/physics/newtonian_hydro.rs:15-28, `Mesh` mirrors src/mesh.rs:84-113,
`Control` mirrors src/app.rs:110-145. Field names are the YAML keys of the
reference's setups/*.yaml, so a parsed setup maps onto these one to one.
Validation follows RelativisticHydro::validate (relativistic_hydro.rs:46-54)
and Mesh::validate (mesh.rs:273-299).
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field, fields
from typing import Optional

from . import abi

RK_ORDERS = {"RK1": 1, "RK2": 2, "RK3": 3}
RIEMANN = {"HLLE": abi.KNC_RIEMANN_HLLE, "HLLC": abi.KNC_RIEMANN_HLLC}
LIGHT_SPEED = 3e10  # src/physics/mod.rs:7


class ConfigError(ValueError):
    pass


def _check_unknown(cls, d: dict):
    known = {f.name for f in fields(cls)}
    extra = set(d) - known
    if extra:  # serde(deny_unknown_fields)
        raise ConfigError(f"unknown field(s) {sorted(extra)} for {cls.__name__}")


@dataclass
class RelativisticHydro:
    gamma_law_index: float
    plm_theta: float
    cfl_number: float
    runge_kutta_order: str
    riemann_solver: str
    adaptive_time_step: bool = False

    system = abi.KNC_SYSTEM_RELATIVISTIC

    def validate(self):
        if not 1.0 <= self.plm_theta <= 2.0:
            raise ConfigError("plm_theta must be in the range [1, 2]")
        if not 0.0 <= self.cfl_number <= 0.7:
            raise ConfigError("cfl_number must be in the range [0.0, 0.7]")
        if self.runge_kutta_order not in RK_ORDERS:
            raise ConfigError(f"runge_kutta_order must be one of {list(RK_ORDERS)}")
        if self.riemann_solver not in RIEMANN:
            raise ConfigError(f"riemann_solver must be one of {list(RIEMANN)}")

    def to_c(self) -> abi.HydroParams:
        self.validate()
        return abi.HydroParams(system=self.system,
                               runge_kutta_order=RK_ORDERS[self.runge_kutta_order],
                               riemann_solver=RIEMANN[self.riemann_solver],
                               adaptive_time_step=int(bool(self.adaptive_time_step)),
                               gamma_law_index=float(self.gamma_law_index),
                               plm_theta=float(self.plm_theta),
                               cfl_number=float(self.cfl_number))

    @classmethod
    def from_dict(cls, d: dict):
        _check_unknown(cls, d)
        return cls(**d)


@dataclass
class NewtonianHydro:
    gamma_law_index: float
    plm_theta: float
    cfl_number: float
    runge_kutta_order: str
    # Extension: the reference's Newtonian adapter is HLLE only
    # (newtonian_hydro.rs:96-102); HLLC selects a Toro HLLC flux.
    riemann_solver: str = "HLLE"

    system = abi.KNC_SYSTEM_NEWTONIAN

    def validate(self):
        if not 1.0 <= self.plm_theta <= 2.0:
            raise ConfigError("plm_theta must be in the range [1, 2]")
        if not 0.0 <= self.cfl_number <= 0.7:
            raise ConfigError("cfl_number must be in the range [0.0, 0.7]")
        if self.runge_kutta_order not in RK_ORDERS:
            raise ConfigError(f"runge_kutta_order must be one of {list(RK_ORDERS)}")
        if self.riemann_solver not in RIEMANN:
            raise ConfigError(f"riemann_solver must be one of {list(RIEMANN)}")

    def to_c(self) -> abi.HydroParams:
        self.validate()
        return abi.HydroParams(system=self.system,
                               runge_kutta_order=RK_ORDERS[self.runge_kutta_order],
                               riemann_solver=RIEMANN[self.riemann_solver],
                               adaptive_time_step=1,
                               gamma_law_index=float(self.gamma_law_index),
                               plm_theta=float(self.plm_theta),
                               cfl_number=float(self.cfl_number))

    @classmethod
    def from_dict(cls, d: dict):
        _check_unknown(cls, d)
        return cls(**d)


@dataclass
class Mesh:
    reference_radius: float
    inner_radius: float
    outer_radius: float
    inner_excision_speed: float
    outer_excision_speed: float
    num_polar_zones: int
    block_size: int
    num_radial_zones: Optional[int] = None
    excision_delay: Optional[float] = None

    def outer_excision_surface(self, t: float) -> float:
        t0 = self.excision_delay or 0.0
        return self.outer_radius + max(t - t0, 0.0) * self.outer_excision_speed

    def inner_excision_surface(self, t: float) -> float:
        t0 = self.excision_delay or 0.0
        return self.inner_radius + max(t - t0, 0.0) * self.inner_excision_speed

    def validate(self, time: float = 0.0):
        if self.reference_radius <= 0.0 or self.inner_radius < 0.0 or self.outer_radius < 0.0:
            raise ConfigError("all radii must be positive")
        if self.reference_radius > self.outer_excision_surface(time):
            raise ConfigError("the reference radius is outside the outer excision surface")
        if (self.excision_delay or 0.0) < 0.0:
            raise ConfigError("the excision delay time must be non-negative")
        if self.inner_excision_speed < 0.0 or self.outer_excision_speed < 0.0:
            raise ConfigError("the excision surface speeds must be non-negative")
        if self.outer_excision_speed < self.inner_excision_speed:
            raise ConfigError("outer_excision_speed < inner_excision_speed "
                              "(the IES would eventually overtake the OES)")
        if self.block_size < 2:
            raise ConfigError("must have at least 2 radial zones per block")
        if self.num_polar_zones != 1 and self.num_polar_zones < 16:
            raise ConfigError("must have at least 16 polar zones")
        if self.num_polar_zones == 1 and self.num_radial_zones is None:
            raise ConfigError("num_radial_zones is not optional when num_polar_zones=1")

    def zone_dlogr(self) -> float:
        if self.num_radial_zones is not None:
            return 1.0 / self.num_radial_zones
        return math.pi / self.num_polar_zones

    def block_dlogr(self) -> float:
        return self.block_size * self.zone_dlogr()

    def block_radii(self, index: int):
        b = 1.0 + self.block_dlogr()
        return (self.reference_radius * b ** index, self.reference_radius * b ** (index + 1))

    def grid_block_indexes(self, time: float = 0.0):
        out = []
        i = 0
        while self.block_radii(i)[0] < self.outer_excision_surface(time):
            out.append(i)
            i += 1
        return out

    def to_c(self) -> abi.MeshParams:
        return abi.MeshParams(
            reference_radius=float(self.reference_radius),
            inner_radius=float(self.inner_radius),
            outer_radius=float(self.outer_radius),
            inner_excision_speed=float(self.inner_excision_speed),
            outer_excision_speed=float(self.outer_excision_speed),
            excision_delay=float(self.excision_delay or 0.0),
            num_radial_zones=int(self.num_radial_zones or 0),
            num_polar_zones=int(self.num_polar_zones),
            block_size=int(self.block_size),
            has_num_radial_zones=int(self.num_radial_zones is not None),
            has_excision_delay=int(self.excision_delay is not None))

    @classmethod
    def from_dict(cls, d: dict):
        _check_unknown(cls, d)
        return cls(**d)


@dataclass
class Control:
    start_time: float
    final_time: float
    checkpoint_interval: float
    fold: int
    products_interval: Optional[float] = None
    num_threads: Optional[int] = None
    snappy_compression: bool = False
    output_directory: str = "."

    @classmethod
    def from_dict(cls, d: dict):
        _check_unknown(cls, d)
        return cls(**d)


# ---- device models -------------------------------------------------------
@dataclass
class WindModel:
    """Cold radial wind: rho = rho0 r^-2 (1 + noise U[0,1)), u^r const, p = T rho."""
    rho0: float = 1.0
    ur: float = 1.0
    temperature: float = 1e-4
    noise: float = 0.01
    seed: int = 1

    def to_c(self) -> abi.ModelParams:
        m = abi.ModelParams(kind=abi.KNC_MODEL_WIND, seed=self.seed)
        m.p[0], m.p[1], m.p[2], m.p[3] = self.rho0, self.ur, self.temperature, self.noise
        return m


@dataclass
class JetModel:
    """Static ambient rho0 r^-2 (seeded noise) and a W = lorentz nozzle inside
    `injection_radius` within `theta_jet` of either pole."""
    rho0: float = 1.0
    temperature: float = 1e-3
    noise: float = 0.01
    theta_jet: float = 0.1
    lorentz: float = 100.0
    density_ratio: float = 1.0
    injection_radius: float = 1.0
    seed: int = 1

    def to_c(self) -> abi.ModelParams:
        m = abi.ModelParams(kind=abi.KNC_MODEL_JET, seed=self.seed)
        vals = [self.rho0, self.temperature, self.noise, self.theta_jet, self.lorentz,
                self.density_ratio, self.injection_radius]
        for k, v in enumerate(vals):
            m.p[k] = v
        return m


@dataclass
class SphereModel:
    """Newtonian over-dense sphere at rest: rho_in inside radius, rho_out outside."""
    rho_in: float = 10.0
    rho_out: float = 1.0
    radius: float = 2.0
    pressure: float = 1e-2
    noise: float = 0.01
    seed: int = 1

    def to_c(self) -> abi.ModelParams:
        m = abi.ModelParams(kind=abi.KNC_MODEL_SPHERE, seed=self.seed)
        for k, v in enumerate([self.rho_in, self.rho_out, self.radius, self.pressure, self.noise]):
            m.p[k] = v
        return m


# ---- the reference's setups, evaluated on the device ---------------------
def _pack(kind, values):
    m = abi.ModelParams(kind=kind, seed=0)
    for k, v in enumerate(values):
        m.p[k] = float(v)
    return m


@dataclass
class JetInCloud:
    """src/models/jet_in_cloud.rs:16-49 (field names as in setups/jet_in_cloud.yaml)."""
    cloud_mass: float
    engine_delay: float
    engine_duration: float
    engine_strength: float
    engine_theta: float
    engine_u: float
    envelop_m1: float
    envelop_slowest_beta: float
    envelop_fastest_beta: float
    envelop_psi: float

    def to_c(self):
        return _pack(abi.KNC_MODEL_JET_IN_CLOUD, [getattr(self, f.name) for f in fields(self)])


@dataclass
class KineticBomb:
    """src/models/kinetic_bomb.rs:12-20."""
    external_medium_density: float
    launch_radius: float
    shell_thickness: float
    kinetic_energy: float
    shell_mass: float

    def to_c(self):
        return _pack(abi.KNC_MODEL_KINETIC_BOMB, [getattr(self, f.name) for f in fields(self)])


@dataclass
class JetInStar:
    """src/models/jet_in_star.rs:36-62."""
    star_mass: float
    engine_duration: float
    engine_energy: float
    engine_theta: float
    engine_u: float
    envelope_radius: float
    envelope_mass: float
    volume_factor: float

    def to_c(self):
        return _pack(abi.KNC_MODEL_JET_IN_STAR, [getattr(self, f.name) for f in fields(self)])


SETUP_MODELS = {"jet_in_cloud": JetInCloud, "kinetic_bomb": KineticBomb, "jet_in_star": JetInStar,
                "wind": WindModel, "jet": JetModel, "sphere": SphereModel}
