"""Named synthetic workloads (hydro, mesh, model, steps).

Each builder returns the configuration of one grid used by the tests and by
bench.py. Block layouts come out of the reference's own mesh rule
(Mesh::subgrid_extent, src/mesh.rs:358-372): block i spans
r_ref (1 + B)^i .. r_ref (1 + B)^(i+1) with B = block_size / num_radial_zones,
so "r in [1, 10]" is realised as the nearest whole number of blocks.
"""
from __future__ import annotations

import random
from dataclasses import dataclass
from typing import Optional

from .config import JetModel, Mesh, NewtonianHydro, RelativisticHydro, SphereModel, WindModel


@dataclass
class Workload:
    name: str
    hydro: object
    mesh: Mesh
    model: object
    steps: int
    # uneven blocks: (first index, [nr], [nq]) for knc_set_block_shapes
    shapes: Optional[tuple] = None

    @property
    def num_blocks(self) -> int:
        return len(self.mesh.grid_block_indexes(0.0))

    def shape_of(self, index: int):
        if self.shapes is not None:
            first, nr, nq = self.shapes
            if first <= index < first + len(nr):
                return nr[index - first], nq[index - first]
        return self.mesh.block_size, self.mesh.num_polar_zones

    @property
    def zones(self) -> int:
        return sum(a * b for a, b in map(self.shape_of, self.mesh.grid_block_indexes(0.0)))

    def apply_shapes(self, solver):
        """Register the block shapes with a solver (GPU or oracle) before init."""
        if self.shapes is not None:
            solver.set_block_shapes(*self.shapes)


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


def _uneven_shapes(seed, count, nr_choices, nq_choices):
    rng = random.Random(seed)
    return [rng.choice(nr_choices) for _ in range(count)], [rng.choice(nq_choices) for _ in range(count)]


def _moving_mesh(num_blocks, block_size, num_radial_zones, nq, speed):
    """Excision surfaces moving at `speed` (cm/s): the inner one just below the
    first block's outer edge, the outer one just below the last block's outer
    edge, so blocks retire at the inner end and activate at the outer end
    within the first steps."""
    b = 1.0 + block_size / num_radial_zones
    r_inner = b ** 1 * (1.0 - 1e-3)
    r_outer = b ** num_blocks * (1.0 - 1e-4)
    return Mesh(reference_radius=1.0, inner_radius=r_inner, outer_radius=r_outer,
                inner_excision_speed=speed, outer_excision_speed=speed,
                num_polar_zones=nq, block_size=block_size, num_radial_zones=num_radial_zones)


def uneven(seed: int = 1, num_blocks: int = 96, order: str = "RK3", riemann: str = "HLLE") -> Workload:
    """96 uneven blocks: nr from {32, ..., 512} and nq from {64, 128, 256}
    drawn per block from a seeded generator (mesh defaults 64 x 64, block
    width dlog r = 0.05, r in [1, 108]); SRHD gamma 4/3, PLM 1.5, RK3, CFL 0.4;
    both excision surfaces move at 0.5 c, so blocks retire at the inner end
    and activate at the outer end while it runs. The seeded r^-2 wind."""
    hydro = RelativisticHydro(gamma_law_index=4.0 / 3.0, plm_theta=1.5, cfl_number=0.4,
                              runge_kutta_order=order, riemann_solver=riemann)
    mesh = _moving_mesh(num_blocks, 64, 1280, 64, 0.5 * 3e10)
    extra = 32   # shapes for blocks activated at the outer end
    nr, nq = _uneven_shapes(seed, num_blocks + extra, [32, 64, 128, 256, 512], [64, 128, 256])
    return Workload(f"uneven_{num_blocks}_blocks", hydro, mesh, WindModel(seed=seed), 200,
                    shapes=(0, nr, nq))


def uneven_small(seed: int = 1, order: str = "RK3", riemann: str = "HLLE", moving: bool = True) -> Workload:
    """8 uneven blocks (nr from {16, 32, 64}, nq from {32, 64, 128}, mesh
    defaults 32 x 32, dlog r = 0.2), CPU-checkable; with `moving` both
    excision surfaces move at 0.5 c."""
    hydro = RelativisticHydro(gamma_law_index=4.0 / 3.0, plm_theta=1.5, cfl_number=0.4,
                              runge_kutta_order=order, riemann_solver=riemann)
    if moving:
        mesh = _moving_mesh(8, 32, 160, 32, 0.5 * 3e10)
    else:
        mesh = Mesh(reference_radius=1.0, inner_radius=1.0, outer_radius=1.2 ** 8 * (1.0 - 1e-4),
                    inner_excision_speed=0.0, outer_excision_speed=0.0,
                    num_polar_zones=32, block_size=32, num_radial_zones=160)
    nr, nq = _uneven_shapes(seed, 8 + 8, [16, 32, 64], [32, 64, 128])
    return Workload("uneven_8_blocks", hydro, mesh, WindModel(seed=seed), 30, shapes=(0, nr, nq))


WORKLOADS = {
    "uneven": uneven,
    "uneven_small": uneven_small,
    "wind_small": wind_small,
    "wind_large": wind_large,
    "sphere_small": sphere_small,
    "sphere_large": sphere_large,
    "jet": jet,
    "jet_small": jet_small,
}
