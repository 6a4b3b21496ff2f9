"""Device models of the reference's setups (src/models/*.rs) against the
oracle's restatement, on small grids in cgs units; and the host-callback
model path against the device model it mirrors.

The models call pow / exp / cos, which CUDA and glibc round differently in
the last bit, so these comparisons allow 1e-10 of each field's scale."""
import numpy as np
import pytest

from helpers import field_errors
from knc import config

pytestmark = pytest.mark.gpu
TOL = 1e-10


def _run(hydro, mesh, model, t0, steps, fold):
    import knc
    import knc_oracle
    g = knc.Solver(hydro, mesh)
    g.set_model(model)
    g.init_from_model(t0)
    o = knc_oracle.Oracle(hydro, mesh, threads=8)
    o.set_model(model)
    o.init_from_model(t0)
    assert g.block_indexes() == o.block_indexes()
    assert max(field_errors(g.state(), o.state(), momentum_scale=True)) <= TOL
    for _ in range(steps // fold):
        g.advance(fold)
        o.advance(fold)
        assert g.block_indexes() == o.block_indexes()
    return g, o


def test_kinetic_bomb_one_dimensional():
    hydro = config.RelativisticHydro(1.333, 1.5, 0.3, "RK2", "HLLC", adaptive_time_step=True)
    mesh = config.Mesh(reference_radius=1e18, inner_radius=1e18, outer_radius=2e19, inner_excision_speed=0.0,
                       outer_excision_speed=0.0, num_polar_zones=1, block_size=64, num_radial_zones=64)
    model = config.KineticBomb(external_medium_density=2e-23, launch_radius=1e18, shell_thickness=2e18,
                               kinetic_energy=5e50, shell_mass=1e32)
    g, o = _run(hydro, mesh, model, 0.0, 20, 5)
    assert g.time()[0] == pytest.approx(o.time()[0], rel=1e-13)
    assert max(field_errors(g.state(), o.state(), momentum_scale=True)) <= TOL


def test_jet_in_cloud_moving_excision():
    hydro = config.RelativisticHydro(1.333, 1.5, 0.4, "RK2", "HLLC")
    mesh = config.Mesh(reference_radius=3e8, inner_radius=0.0, outer_radius=0.0, inner_excision_speed=3e8,
                       outer_excision_speed=3e10, num_polar_zones=32, block_size=8)
    model = config.JetInCloud(cloud_mass=5e31, engine_delay=1.0, engine_duration=2.0, engine_strength=0.5,
                              engine_theta=0.15, engine_u=20.0, envelop_m1=1e27, envelop_slowest_beta=0.2,
                              envelop_fastest_beta=0.99, envelop_psi=0.3)
    g, o = _run(hydro, mesh, model, 1.0, 20, 5)
    assert g.time() == o.time()
    assert max(field_errors(g.state(), o.state(), momentum_scale=True)) <= TOL


def test_jet_in_star():
    hydro = config.RelativisticHydro(1.33, 1.5, 0.3, "RK2", "HLLC")
    mesh = config.Mesh(reference_radius=1e9, inner_radius=1e9, outer_radius=1e12, inner_excision_speed=1e9,
                       outer_excision_speed=3e10, num_polar_zones=32, block_size=8, excision_delay=10.0)
    model = config.JetInStar(star_mass=1e34, engine_duration=10.0, engine_energy=1e51, engine_theta=0.1,
                             engine_u=40.0, envelope_radius=1e11, envelope_mass=1e31, volume_factor=1.0)
    g, o = _run(hydro, mesh, model, 0.0, 20, 5)
    assert max(field_errors(g.state(), o.state(), momentum_scale=True)) <= TOL


def test_host_callback_model_equals_device_model():
    """knc_set_host_model (any InitialModel evaluated on the host) gives the
    same run as the device model with the same formulas."""
    import knc
    from knc import workloads
    w = workloads.wind_small()
    w.model.noise = 0.0
    dev = knc.build_solver(w)
    host = knc.Solver(w.hydro, w.mesh)

    def wind(r, q, t):
        rho = 1.0 * (1.0 / (r * r))
        return [1.0, 0.0, rho, 1e-4 * rho], 0.0     # AnyPrimitive [u_r, u_theta, rho, p]

    host.set_host_model(wind)
    host.init_from_model(0.0)
    dev.advance(3)
    host.advance(3)
    sd, sh = dev.state(), host.state()
    for i in sd:
        assert np.array_equal(sd[i][0], sh[i][0]) and np.array_equal(sd[i][1], sh[i][1])
