"""Invariants of the CPU oracle's physics (the checker must itself be right).

The reference ships no known-answer vectors for this path, so the oracle is
held to properties any correct restatement has: prim -> cons -> prim round
trips, F(p, p) = F(p), exact stationary contacts for HLLC, discrete
conservation (the change of total mass equals the flux through the two radial
boundary faces) and equatorial mirror symmetry.
"""
import numpy as np
import pytest

import knc_oracle as ko
from knc import config, workloads


def srhd(riemann="HLLE"):
    return config.RelativisticHydro(4.0 / 3.0, 1.5, 0.4, "RK2", riemann).to_c()


def newt(riemann="HLLE"):
    return config.NewtonianHydro(5.0 / 3.0, 1.5, 0.4, "RK2", riemann).to_c()


def random_srhd_prims(n, seed=0):
    rng = np.random.default_rng(seed)
    W = np.exp(rng.uniform(0, np.log(1000), n))
    T = np.exp(rng.uniform(np.log(1e-6), np.log(100), n))
    rho = np.exp(rng.uniform(np.log(1e-3), np.log(1e3), n))
    ang = rng.uniform(0, 2 * np.pi, n)
    um = np.sqrt(W * W - 1)
    return np.stack([rho, um * np.cos(ang), um * np.sin(ang), T * rho], axis=1)


def test_srhd_round_trip(oracle_lib):
    hp = srhd()
    for P in random_srhd_prims(2000):
        U = ko.prim_to_cons(hp, P)
        kind, Q, it = ko.cons_to_prim(hp, U)
        assert kind == 0 and 1 <= it <= 50
        w2 = 1 + P[1] ** 2 + P[2] ** 2
        # the residual |f| < 1e-12 (D + tau) fixes the velocity to ~W^2 1e-12
        assert np.allclose(Q[:3], P[:3], rtol=1e-11 * w2 + 1e-13, atol=0)
        assert abs(Q[3] - P[3]) <= 1e-11 * (U[0] + U[3])


def test_newtonian_round_trip(oracle_lib):
    hp = newt()
    rng = np.random.default_rng(1)
    for _ in range(500):
        P = np.array([rng.uniform(0.1, 10), rng.normal(), rng.normal(), rng.uniform(0.01, 10)])
        kind, Q, _ = ko.cons_to_prim(hp, ko.prim_to_cons(hp, P))
        assert kind == 0 and np.allclose(Q, P, rtol=1e-13, atol=1e-15)


@pytest.mark.parametrize("system", ["srhd", "newt"])
@pytest.mark.parametrize("riemann", ["HLLE", "HLLC"])
def test_flux_consistency(oracle_lib, system, riemann):
    hp = srhd(riemann) if system == "srhd" else newt(riemann)
    prims = random_srhd_prims(200, seed=2)
    if system == "newt":
        prims[:, 1:3] = np.tanh(prims[:, 1:3] / 10)
    for P in prims:
        for axis in (0, 1):
            f, _, _ = ko.flux(hp, P, axis)
            g = ko.riemann(hp, P, P, 0.3, 0.3, axis)
            assert np.allclose(g[:4], f, rtol=1e-12, atol=1e-12 * np.abs(f).max()), (P, axis)


@pytest.mark.parametrize("system", ["srhd", "newt"])
def test_hllc_keeps_stationary_contact(oracle_lib, system):
    hp = srhd("HLLC") if system == "srhd" else newt("HLLC")
    he = srhd("HLLE") if system == "srhd" else newt("HLLE")
    pl = np.array([1.0, 0.0, 0.0, 0.1])
    pr = np.array([0.125, 0.0, 0.0, 0.1])
    for axis in (0, 1):
        f = ko.riemann(hp, pl, pr, 1.0, 0.0, axis)
        expect = np.zeros(4)
        expect[1 + axis] = 0.1
        assert np.allclose(f[:4], expect, atol=1e-15) and abs(f[4]) < 1e-15
        fe = ko.riemann(he, pl, pr, 1.0, 0.0, axis)
        assert abs(fe[0]) > 1e-3      # HLLE diffuses the contact


def test_plm_gradient(oracle_lib):
    assert ko.plm_gradient(1.5, 0.0, 1.0, 2.0) == 1.0
    assert ko.plm_gradient(1.5, 0.0, 1.0, 1.2) == pytest.approx(0.3)
    assert ko.plm_gradient(1.5, 0.0, 1.0, 0.5) == 0.0
    assert ko.plm_gradient(1.0, 2.0, 1.0, 0.0) == -1.0


def test_geometry_sums(oracle_lib):
    w = workloads.wind_small()
    mp = w.mesh.to_c()
    total = 0.0
    for i in w.mesh.grid_block_indexes():
        g = ko.block_geometry(mp, i)
        total += g["dv"].sum()
        r0, r1 = g["rv"][0], g["rv"][-1]
        assert g["dv"].sum() == pytest.approx(4 * np.pi / 3 * (r1 ** 3 - r0 ** 3), rel=1e-12)
        # face areas of a radial shell: the frustum areas approach 4 pi r^2
        assert g["ar"][0].sum() == pytest.approx(4 * np.pi * r0 ** 2, rel=1e-3)
        assert np.all(g["ar"] > 0) and np.all(g["aq"][:, 1:-1] > 0)
    assert total > 0


def _prims(hp, cons, dv):
    out = np.empty(cons.shape[:2] + (4,))
    for i in range(cons.shape[0]):
        for j in range(cons.shape[1]):
            kind, p, _ = ko.cons_to_prim(hp, cons[i, j] / dv[i, j])
            assert kind in (0, 2)
            out[i, j] = p
    return out


def test_discrete_conservation_rk1(oracle_lib):
    """One Euler stage: sum of D dV changes by exactly -dt c sum(F_D A) over the
    inner and outer boundary faces (polar faces are closed at the poles)."""
    w = workloads.wind_small()
    w.mesh.num_polar_zones = 16
    w.hydro.runge_kutta_order = "RK1"
    hp, mp = w.hydro.to_c(), w.mesh.to_c()
    o = ko.Oracle(w.hydro, w.mesh, threads=4)
    o.set_model(w.model)
    o.init_from_model(0.0)
    idx = o.block_indexes()
    st0 = o.state()
    dt = o.time_step()
    o.advance(1)
    st1 = o.state()
    m0 = sum(st0[i][0][..., 0].sum() for i in idx)
    m1 = sum(st1[i][0][..., 0].sum() for i in idx)
    th = w.hydro.plm_theta

    def ghost_rows(index, rows):
        g = ko.block_geometry(mp, index)
        out = []
        for i in rows:
            row = []
            for j in range(w.mesh.num_polar_zones):
                r = g["rc"][i, j]
                rho = 1.0 / (r * r)
                p = np.array([rho, 1.0, 0.0, 1e-4 * rho])
                U = ko.prim_to_cons(hp, p) * g["dv"][i, j]
                row.append(ko.cons_to_prim(hp, U / g["dv"][i, j])[1])
            out.append(row)
        return np.array(out)

    def face_flux(pe, area):
        # pe: 4 rows of prims around the face (two left, two right) -> mass flux x area
        tot = 0.0
        for j in range(pe.shape[1]):
            gl = [ko.plm_gradient(th, pe[0, j, q], pe[1, j, q], pe[2, j, q]) for q in range(4)]
            gr = [ko.plm_gradient(th, pe[1, j, q], pe[2, j, q], pe[3, j, q]) for q in range(4)]
            pl = pe[1, j] + 0.5 * np.array(gl)
            pr = pe[2, j] - 0.5 * np.array(gr)
            f = ko.riemann(hp, pl, pr, 0.0, 0.0, 0)
            tot += f[0] * 3e10 * area[j]
        return tot

    g_in = ko.block_geometry(mp, idx[0])
    g_out = ko.block_geometry(mp, idx[-1])
    p_in = _prims(hp, st0[idx[0]][0][:2], g_in["dv"][:2])
    p_out = _prims(hp, st0[idx[-1]][0][-2:], g_out["dv"][-2:])
    gh_in = ghost_rows(idx[0] - 1, [w.mesh.block_size - 2, w.mesh.block_size - 1])
    gh_out = ghost_rows(idx[-1] + 1, [0, 1])
    f_in = face_flux(np.concatenate([gh_in, p_in]), g_in["ar"][0])
    f_out = face_flux(np.concatenate([p_out, gh_out]), g_out["ar"][-1])
    expected = -(f_out - f_in) * dt
    assert (m1 - m0) == pytest.approx(expected, rel=1e-9, abs=1e-12 * m0)


def test_equatorial_mirror_symmetry(oracle_lib):
    w = workloads.jet_small()
    w.model.noise = 0.0
    o = ko.Oracle(w.hydro, w.mesh, threads=4)
    o.set_model(w.model)
    o.init_from_model(0.0)
    o.advance(20)
    for i, (cons, scal) in o.state().items():
        mir = cons[:, ::-1, :]
        for q, sign in [(0, 1), (1, 1), (2, -1), (3, 1)]:
            # S_theta is judged on the momentum scale (it is round-off where the flow is radial)
            scale = np.abs(cons[..., 1:3] if q == 2 else cons[..., q]).max() + 1e-300
            assert np.abs(cons[..., q] - sign * mir[..., q]).max() <= 1e-10 * scale, (i, q)
        assert np.abs(scal - scal[:, ::-1]).max() <= 1e-10 * (np.abs(scal).max() + 1e-300)
