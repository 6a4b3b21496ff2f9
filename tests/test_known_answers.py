"""Known-answer tests of the CPU oracle's scheme (the reference ships none).

- Shock tubes against exact Riemann solutions computed by the test's own
  solvers (`exact_riemann.py`): Newtonian and special-relativistic ideal
  gases, HLLE and HLLC, PLM 1.5, RK2. A tube is a thin radial shell far from
  the origin (r in [1e6, 1e6 + 2] cm, one polar zone), planar to ~1e-6; its
  ends take the sphere model's states, and the comparison window (the middle
  half) is one the end waves do not reach in the run time. The density's L1
  error there must be small and fall under refinement (first order at the
  discontinuities).
- A uniform static state on the spherical grid: the scheme's radial face
  areas (frusta) and centroid sources do not balance exactly, so the gas
  starts to move; the velocity reached by a fixed time must fall at second
  order when the grid is refined in both directions.
"""
import math

import numpy as np
import pytest

import knc_oracle as ko
from exact_riemann import Newtonian, Relativistic, srhd_conserved
from knc import config, workloads

LIGHT_SPEED = 3e10


# ---- the exact solvers themselves ------------------------------------------
@pytest.mark.parametrize("left,right,gamma", [((1.0, 0.0, 2.0), (0.2, 0.0, 0.1), 5.0 / 3.0),
                                              ((5.0, 0.0, 10.0), (1.0, 0.0, 1e-5), 5.0 / 3.0),
                                              ((1.0, 0.5, 1.0), (1.0, -0.5, 1.0), 5.0 / 3.0),
                                              ((1.0, 0.0, 1.0), (0.3, 0.2, 3.0), 4.0 / 3.0)])
def test_srhd_exact_solution_is_consistent(left, right, gamma):
    """Shocks satisfy the jump conditions F_b - F_a = V_s (U_b - U_a) in the
    lab frame; across fans the Riemann invariant is constant and the
    characteristic speed equals x/t; both sides of the contact share (v, p)."""
    ex = Relativistic(left, right, gamma)
    sg = math.sqrt(gamma - 1.0)
    for a, s in ((left, -1.0), (right, 1.0)):
        if ex.ps > a[2]:
            rho_b, v_b, Vs = ex.shock(a, ex.ps, s)
            assert v_b == pytest.approx(ex.vs, rel=1e-9, abs=1e-12)
            Ua, Fa = srhd_conserved(gamma, *a)
            Ub, Fb = srhd_conserved(gamma, rho_b, v_b, ex.ps)
            scale = np.abs(Fa).max() + np.abs(Fb).max()
            assert np.abs((Fb - Fa) - Vs * (Ub - Ua)).max() <= 1e-12 * scale
        else:
            def J(rho, v, p):
                c = math.sqrt(gamma * p / (rho * (1.0 + gamma / (gamma - 1.0) * p / rho)))
                return 0.5 * math.log((1.0 + v) / (1.0 - v)) + s * (-1.0 / sg) * math.log((sg + c) / (sg - c))
            j0 = J(*a)
            for p in np.geomspace(ex.ps, a[2], 7):
                rho, v = ex.rarefaction(a, p, s)
                assert J(rho, v, p) == pytest.approx(j0, abs=1e-12)
    assert ex.v_after(left, ex.ps, -1.0) == pytest.approx(ex.v_after(right, ex.ps, 1.0), abs=1e-12)


def test_newtonian_exact_solution_is_consistent():
    """Mass and momentum jump conditions across the shock; constant state in
    the star region; the fan joins the left state to the star state."""
    g = 1.4
    left, right = (1.0, 0.0, 1.0), (0.2, 0.0, 0.15)
    ex = Newtonian(left, right, g)
    cr = math.sqrt(g * right[2] / right[0])
    S = cr * math.sqrt((g + 1.0) / (2.0 * g) * ex.ps / right[2] + (g - 1.0) / (2.0 * g))
    rho_b, u_b, p_b = ex.sample(S * (1.0 - 1e-9))
    assert rho_b * (u_b - S) == pytest.approx(right[0] * (0.0 - S), rel=1e-12)
    assert rho_b * u_b * (u_b - S) + p_b == pytest.approx(right[2], rel=1e-12)
    cl = math.sqrt(g * left[2] / left[0])
    assert ex.sample(-cl * (1.0 + 1e-9)) == left
    tail = ex.us - cl * (ex.ps / left[2]) ** ((g - 1.0) / (2.0 * g))
    fan_end = ex.sample(tail * (1.0 + 1e-9))
    assert fan_end[1] == pytest.approx(ex.us, rel=1e-6) and fan_end[2] == pytest.approx(ex.ps, rel=1e-6)


# ---- shock tubes through the oracle's scheme ---------------------------------
R0 = 1e6            # cm: the tube's inner end
BLOCK = 0.5 / R0    # block width in log r: 4 blocks make a 2 cm tube


def _tube(system, riemann, zones_per_block, left, right, gamma, t_end, make=None, out=None):
    """Run a shock tube in the oracle (or in the solver `make(hydro, mesh)`
    returns); density L1 error against the exact solution over the middle
    half of the tube, at the time reached. `out` receives the final
    primitives per block."""
    nb = 4
    mesh = config.Mesh(reference_radius=R0, inner_radius=R0, outer_radius=R0 * (1 + BLOCK) ** nb * (1 - 1e-12),
                       inner_excision_speed=0.0, outer_excision_speed=0.0, num_polar_zones=1,
                       block_size=zones_per_block, num_radial_zones=int(round(zones_per_block / BLOCK)))
    if system == "newtonian":
        hydro = config.NewtonianHydro(gamma, 1.5, 0.4, "RK2", riemann)
    else:
        hydro = config.RelativisticHydro(gamma, 1.5, 0.4, "RK2", riemann)
    hp, mp = hydro.to_c(), mesh.to_c()
    x0 = R0 * ((1 + BLOCK) ** nb - 1) / 2     # the diaphragm, mid-tube
    o = make(hydro, mesh) if make else ko.Oracle(hydro, mesh, threads=1)
    o.set_model(config.SphereModel(rho_in=left[0], rho_out=right[0], radius=R0 + x0, pressure=right[2],
                                   noise=0.0))
    o.init_from_model(0.0)
    idx = o.block_indexes()
    assert len(idx) == nb
    geo = {i: ko.block_geometry(mp, i) for i in idx}
    for i in idx:
        g = geo[i]
        cons = np.empty((zones_per_block, 1, 4))
        for k in range(zones_per_block):
            rho, v, p = left if g["rc"][k, 0] - R0 < x0 else right
            u = v / math.sqrt(1.0 - v * v) if system == "srhd" else v   # four-velocity for SRHD
            cons[k, 0] = ko.prim_to_cons(hp, np.array([rho, u, 0.0, p])) * g["dv"][k, 0]
        o.add_block(i, cons, np.zeros((zones_per_block, 1)))
    while o.time()[0] < t_end * (1.0 - 1e-12):
        o.advance(1)
    t = o.time()[0]
    x = np.concatenate([geo[i]["rc"][:, 0] - R0 - x0 for i in idx])
    prims = {i: o.get_primitives(i) for i in idx}
    if out is not None:
        out.update(prims)
    rho = np.concatenate([prims[i][:, 0, 0] for i in idx])
    ex = Newtonian(left, right, gamma) if system == "newtonian" else Relativistic(left, right, gamma)
    xi = x / (t if system == "newtonian" else t * LIGHT_SPEED)
    exact = np.array([ex.sample(z)[0] for z in xi])
    window = np.abs(x) < 0.5 * x0
    return np.abs(rho - exact)[window].mean()


TUBES = {
    # system, left (rho, v, p), right, gamma, end time, L1 bound at 800 zones
    "newtonian": ("newtonian", (1.0, 0.0, 1.0), (0.2, 0.0, 0.15), 1.4, 0.2, 2.1e-3),
    "srhd_mild": ("srhd", (1.0, 0.0, 2.0), (0.2, 0.0, 0.1), 5.0 / 3.0, 0.4 / LIGHT_SPEED, 3.3e-3),
    "srhd_blast": ("srhd", (5.0, 0.0, 10.0), (1.0, 0.0, 1e-5), 5.0 / 3.0, 0.4 / LIGHT_SPEED, 0.055),
    "srhd_collision": ("srhd", (1.0, 0.5, 1.0), (1.0, -0.5, 1.0), 5.0 / 3.0, 0.4 / LIGHT_SPEED, 9e-3),
}


@pytest.mark.parametrize("riemann", ["HLLE", "HLLC"])
@pytest.mark.parametrize("name", list(TUBES))
def test_shock_tube_against_exact_solution(oracle_lib, name, riemann):
    system, left, right, gamma, t_end, bound = TUBES[name]
    coarse = _tube(system, riemann, 100, left, right, gamma, t_end)
    fine = _tube(system, riemann, 200, left, right, gamma, t_end)
    assert fine < bound, (coarse, fine)
    assert fine < 0.65 * coarse, (coarse, fine)


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["newtonian", "srhd_blast"])
def test_gpu_shock_tube_bitwise(oracle_lib, name):
    """The FP64 GPU stage through the C ABI on the same tubes: primitives
    bit for bit the oracle's, so the same L1 against the exact solution."""
    import knc
    system, left, right, gamma, t_end, bound = TUBES[name]
    po, pg = {}, {}
    l1o = _tube(system, "HLLC", 200, left, right, gamma, t_end, out=po)
    l1g = _tube(system, "HLLC", 200, left, right, gamma, t_end, make=knc.Solver, out=pg)
    assert l1g == l1o and l1g < bound
    for i in po:
        assert np.array_equal(pg[i], po[i]), i


# ---- uniform static state ------------------------------------------------------
@pytest.mark.parametrize("system", ["newtonian", "srhd"])
def test_uniform_static_state_imbalance_converges(oracle_lib, system):
    """Uniform rho = 1, p = 1e-2 at rest on r in [1, 10] (4 blocks): max |u|
    over the sound speed at a fixed time falls ~4x per doubling of both
    resolutions (16, 32, 64 polar zones and rows per block)."""
    if system == "newtonian":
        gamma, T = 5.0 / 3.0, 2.0
        cs = math.sqrt(gamma * 1e-2)
    else:
        gamma, T = 4.0 / 3.0, 1e-11
        cs = math.sqrt(gamma * 1e-2 / (1.0 + gamma / (gamma - 1.0) * 1e-2))
    vmax = []
    for n, nrz in ((16, 20), (32, 41), (64, 82)):
        w = workloads.wind_small()
        w.mesh.num_polar_zones, w.mesh.block_size, w.mesh.num_radial_zones = n, n, nrz
        hydro = (config.NewtonianHydro(gamma, 1.5, 0.4, "RK2", "HLLE") if system == "newtonian"
                 else config.RelativisticHydro(gamma, 1.5, 0.4, "RK2", "HLLE"))
        o = ko.Oracle(hydro, w.mesh, threads=4)
        o.set_model(config.SphereModel(rho_in=1.0, rho_out=1.0, radius=0.5, pressure=1e-2, noise=0.0))
        o.init_from_model(0.0)
        while o.time()[0] < T:
            o.advance(1)
        vmax.append(max(np.abs(o.get_primitives(i)[..., 1:3]).max() for i in o.block_indexes()) / cs)
    assert vmax[2] < 2e-4
    assert vmax[0] / vmax[1] > 3.5 and vmax[1] / vmax[2] > 3.5, vmax
