"""Named synthetic workloads (hydro, mesh, model, steps).

Each builder returns the configuration of one grid used by the tests and by
bench.py. Block layouts come out of the reference's own mesh rule
(Mesh::subgrid_extent, src/mesh.rs:358-372): block i spans
r_ref (1 + B)^i .. r_ref (1 + B)^(i+1) with B = block_size / num_radial_zones,
so "r in [1, 10]" is realised as the nearest whole number of blocks.
"""
from __future__ import annotations

from dataclasses import dataclass

from .config import JetModel, Mesh, NewtonianHydro, RelativisticHydro, SphereModel, WindModel


@dataclass
class Workload:
    name: str
    hydro: object
    mesh: Mesh
    model: object
    steps: int

    @property
    def num_blocks(self) -> int:
        return len(self.mesh.grid_block_indexes(0.0))

    @property
    def zones(self) -> int:
        return self.num_blocks * self.mesh.block_size * self.mesh.num_polar_zones


def wind_small(seed: int = 1) -> Workload:
    """4 blocks of 64 x 128 over r in [1, 10.05]: SRHD gamma 4/3, PLM 1.5,
    HLLE, RK2, CFL 0.4, fixed excision, 100 steps."""
    hydro = RelativisticHydro(gamma_law_index=4.0 / 3.0, plm_theta=1.5, cfl_number=0.4,
                              runge_kutta_order="RK2", riemann_solver="HLLE")
    mesh = Mesh(reference_radius=1.0, inner_radius=1.0, outer_radius=10.0,
                inner_excision_speed=0.0, outer_excision_speed=0.0,
                num_polar_zones=128, block_size=64, num_radial_zones=82)
    return Workload("wind_4x64x128", hydro, mesh, WindModel(seed=seed), 100)


def wind_large(seed: int = 1) -> Workload:
    """64 blocks of 64 x 1024 (4096 x 1024 zones) over r in [1, 10.0008]:
    the same wind, FP64, 200 steps."""
    hydro = RelativisticHydro(gamma_law_index=4.0 / 3.0, plm_theta=1.5, cfl_number=0.4,
                              runge_kutta_order="RK2", riemann_solver="HLLE")
    mesh = Mesh(reference_radius=1.0, inner_radius=1.0, outer_radius=10.0,
                inner_excision_speed=0.0, outer_excision_speed=0.0,
                num_polar_zones=1024, block_size=64, num_radial_zones=1747)
    return Workload("wind_64x64x1024", hydro, mesh, WindModel(seed=seed), 200)


def sphere_large(seed: int = 1, riemann: str = "HLLE") -> Workload:
    """Newtonian gamma 5/3 over-dense sphere on the 4096 x 1024 grid."""
    hydro = NewtonianHydro(gamma_law_index=5.0 / 3.0, plm_theta=1.5, cfl_number=0.4,
                           runge_kutta_order="RK2", riemann_solver=riemann)
    mesh = Mesh(reference_radius=1.0, inner_radius=1.0, outer_radius=10.0,
                inner_excision_speed=0.0, outer_excision_speed=0.0,
                num_polar_zones=1024, block_size=64, num_radial_zones=1747)
    return Workload(f"sphere_{riemann.lower()}_64x64x1024", hydro, mesh, SphereModel(seed=seed), 200)


def sphere_small(seed: int = 1, riemann: str = "HLLE") -> Workload:
    hydro = NewtonianHydro(gamma_law_index=5.0 / 3.0, plm_theta=1.5, cfl_number=0.4,
                           runge_kutta_order="RK2", riemann_solver=riemann)
    mesh = Mesh(reference_radius=1.0, inner_radius=1.0, outer_radius=10.0,
                inner_excision_speed=0.0, outer_excision_speed=0.0,
                num_polar_zones=128, block_size=64, num_radial_zones=82)
    return Workload(f"sphere_{riemann.lower()}_4x64x128", hydro, mesh, SphereModel(seed=seed), 100)


def jet(seed: int = 1, nq: int = 512, num_radial_zones: int = 857) -> Workload:
    """Relativistic jet (W = 100, theta_j = 0.1, p/rho = 1e-3) injected through
    r = 1 into a seeded r^-2 ambient: 32 blocks of 64 x 512 (2048 x 512)."""
    hydro = RelativisticHydro(gamma_law_index=4.0 / 3.0, plm_theta=1.5, cfl_number=0.4,
                              runge_kutta_order="RK2", riemann_solver="HLLE")
    mesh = Mesh(reference_radius=1.0, inner_radius=1.0, outer_radius=10.0,
                inner_excision_speed=0.0, outer_excision_speed=0.0,
                num_polar_zones=nq, block_size=64, num_radial_zones=num_radial_zones)
    return Workload(f"jet_{nq}", hydro, mesh, JetModel(seed=seed), 200)


def jet_small(seed: int = 1) -> Workload:
    """The jet on 4 blocks of 64 x 128 (CPU-checkable)."""
    w = jet(seed=seed, nq=128, num_radial_zones=82)
    w.name = "jet_4x64x128"
    w.steps = 100
    return w


WORKLOADS = {
    "wind_small": wind_small,
    "wind_large": wind_large,
    "sphere_small": sphere_small,
    "sphere_large": sphere_large,
    "jet": jet,
    "jet_small": jet_small,
}
