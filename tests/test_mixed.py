"""The mixed-precision stage: FP32 reconstruction / flux / sources, FP64
state accumulation and FP64 recovery above the Lorentz-factor split.
Accuracy is reported per field against the FP64 oracle (L1 relative to the
field's L1 norm, and max difference relative to the field's max)."""
import numpy as np
import pytest

from helpers import field_errors, make_pair

pytestmark = pytest.mark.gpu


def l1_errors(a, b):
    out = []
    for q in range(5):
        num = den = 0.0
        for k in b:
            x = a[k][0][..., q] if q < 4 else a[k][1]
            y = b[k][0][..., q] if q < 4 else b[k][1]
            num += float(np.abs(x - y).sum())
            den += float(np.abs(y).sum())
        out.append(num / den if den else num)
    return out


def _mixed_vs_oracle(workload, steps, w_split=2.0):
    from knc import abi
    g, o = make_pair(workload)
    g.set_precision(abi.KNC_PRECISION_MIXED)
    g.set_mixed_w_split(w_split)
    g.advance(steps)
    o.advance(steps)
    return g, o, l1_errors(g.state(), o.state()), field_errors(g.state(), o.state())


def test_wind_l1_density_below_1e6():
    from knc import workloads
    w = workloads.wind_small()
    g, o, l1, linf = _mixed_vs_oracle(w, w.steps)
    print("wind L1", l1, "max", linf)
    for q in (0, 1, 3):            # D, S_r, tau (S_theta and the scalar are ~0 here)
        assert l1[q] <= 1e-6, (q, l1)
        assert linf[q] <= 1e-5, (q, linf)
    assert g.time() == o.time()


def _comoving_density_l1(g, o):
    num = den = 0.0
    for i in o.block_indexes():
        a = g.get_primitives(i)[..., 0]
        b = o.get_primitives(i)[..., 0]
        num += float(np.abs(a - b).sum())
        den += float(np.abs(b).sum())
    return num / den


def test_jet_density_l1_below_1e6():
    """The W = 100 jet, the mixed-precision configuration: density L1 against
    the FP64 oracle after 100 steps at most 1e-6, both for the lab-frame
    density D (volume integrals) and for the comoving density rho per zone.
    Faces whose stencil reaches a zone above the Lorentz-factor split are
    solved in FP64; with FP32 faces everywhere rho L1 is 3e-5."""
    from knc import workloads
    w = workloads.jet_small()
    g, o, l1, linf = _mixed_vs_oracle(w, w.steps)
    rho = _comoving_density_l1(g, o)
    print("jet L1", l1, "max", linf, "rho L1", rho)
    assert l1[0] <= 1e-6, l1
    assert rho <= 1e-6, rho
    assert max(linf) <= 1e-4, linf
    assert g.time() == o.time()


def test_jet_fp64_faces_follow_the_split():
    """The FP64 faces follow the Lorentz-factor split: with the split above
    every zone's W the jet runs on FP32 faces alone and its density error
    is FP32's (well above 1e-6); at the default split it is below 1e-6."""
    from knc import workloads
    w = workloads.jet_small()
    _, _, l1_fp32, _ = _mixed_vs_oracle(w, 40, w_split=1e4)
    _, _, l1_split, _ = _mixed_vs_oracle(w, 40)
    print("jet D L1 at 40 steps: FP32 faces", l1_fp32[0], "FP64 faces above W = 2", l1_split[0])
    assert l1_split[0] <= 1e-6
    assert l1_fp32[0] >= 10 * l1_split[0]


def test_w_split_selects_recovery_precision():
    from knc import abi, workloads
    w = workloads.wind_small()
    g, _ = make_pair(w, gpu=True)
    g.set_precision(abi.KNC_PRECISION_MIXED)
    g.set_mixed_w_split(1.0)          # every zone recovers in FP64
    g.reset_c2p_stats()
    g.advance(2)
    st = g.c2p_stats()
    assert st["iters_fp64"] >= st["zones"]
    g.set_mixed_w_split(1e9)          # every zone recovers in FP32
    g.reset_c2p_stats()
    g.advance(2)
    st = g.c2p_stats()
    assert st["iters_fp64"] == 0 and st["iters_fp32"] > 0


def test_mixed_graph_equals_mixed_stream():
    from knc import abi, workloads
    w = workloads.wind_small()
    a, _ = make_pair(w, gpu=True)
    b, _ = make_pair(w, gpu=True)
    for s in (a, b):
        s.set_precision(abi.KNC_PRECISION_MIXED)
    b.set_batched(True)
    a.advance(6)
    b.advance(3)
    b.advance(3)
    sa, sb = a.state(), b.state()
    for k in sa:
        assert np.array_equal(sa[k][0], sb[k][0]) and np.array_equal(sa[k][1], sb[k][1])
    assert a.time() == b.time()


def test_fp64_graph_bitwise():
    from knc import workloads
    w = workloads.wind_small()
    g, o = make_pair(w)
    g.set_batched(True)
    g.advance(5)
    o.advance(5)
    assert max(field_errors(g.state(), o.state())) == 0.0


def test_mixed_adaptive_dt_in_the_fold():
    """Mixed precision with adaptive dt: the fold's first (mixed) recovery
    finds dt from FP32 signal speeds; the time stays within 1e-5 of the FP64
    path's and the state stays close."""
    import knc
    from helpers import field_errors, make_pair
    from knc import workloads
    w = workloads.wind_small()
    w.hydro.adaptive_time_step = True
    g64, _ = make_pair(w, gpu=True)
    gm, _ = make_pair(w, gpu=True)
    gm.set_precision(knc.abi.KNC_PRECISION_MIXED)
    gm.set_batched(True)
    for _ in range(3):
        g64.advance(5)
        gm.advance(5)
    t64, tm = g64.time()[0], gm.time()[0]
    assert abs(tm - t64) <= 1e-5 * t64
    errs = field_errors(gm.state(), g64.state())
    assert errs[0] <= 1e-4, errs


def test_mixed_in_cgs_units():
    """The reference's setups are in cgs (radii 1e8-1e19 cm, densities down to
    1e-20 g/cm^3): the mixed stage works in a power-of-two length unit near
    the reference radius and recovers per unit mass, so the same wind at
    r ~ 1e18 cm and rho ~ 1e-20 stays as close to the FP64 path as in code
    units."""
    import dataclasses
    import knc
    from helpers import field_errors, make_pair
    from knc import workloads
    w = workloads.wind_small()
    w.mesh = dataclasses.replace(w.mesh, reference_radius=1e18, inner_radius=1e18, outer_radius=1e19)
    w.model = dataclasses.replace(w.model, rho0=1e16)
    g64, _ = make_pair(w, gpu=True)
    gm, _ = make_pair(w, gpu=True)
    gm.set_precision(knc.abi.KNC_PRECISION_MIXED)
    for _ in range(4):
        g64.advance(5)
        gm.advance(5)
    st = gm.state()
    assert all(np.isfinite(c).all() and np.isfinite(s).all() for c, s in st.values())
    errs = field_errors(st, g64.state(), momentum_scale=True)
    assert max(errs) <= 1e-5, errs


def test_wind_hllc_against_the_oracle():
    """The mixed stage with the relativistic HLLC solver (Mignone & Bodo):
    the same accuracy bar as HLLE against the FP64 oracle."""
    from knc import workloads
    w = workloads.wind_small()
    w.hydro.riemann_solver = "HLLC"
    g, o, l1, linf = _mixed_vs_oracle(w, w.steps)
    for q in (0, 1, 3):
        assert l1[q] <= 1e-6, (q, l1)
        assert linf[q] <= 1e-5, (q, linf)


@pytest.mark.parametrize("riemann,order", [("HLLE", "RK2"), ("HLLC", "RK2"), ("HLLE", "RK3")])
def test_jet_update_forms_agree(riemann, order):
    """Tiles, tensor-copy tiles, warp strips (with the deferred recovery) and
    the fused stage give the same bits on the jet, whose zones above the
    Lorentz-factor split bring in the FP64 faces, with HLLE and HLLC, and
    with RK3, whose middle stage updates the state in place."""
    import knc
    from helpers import zone_relative_errors
    from knc import workloads
    w = workloads.jet_small()
    w.hydro.riemann_solver = riemann
    w.hydro.runge_kutta_order = order
    states = []
    for t in (dict(tile_rows=8), dict(tile_rows=8, tma=True), dict(tile_rows=16, strip=True, deferred=True),
              dict(tile_rows=8, fused=True), dict(tile_rows=16, strip=True, fused=True)):
        g = knc.build_solver(w)
        g.set_precision(knc.abi.KNC_PRECISION_MIXED)
        g.set_tuning(**t)
        g.advance(12)
        states.append(g.state())
    for st in states[1:]:
        assert max(zone_relative_errors(st, states[0])) == 0.0


def test_mixed_refuses_what_it_does_not_cover():
    """The mixed stage is built for relativistic hydro on a polar grid: a
    Newtonian context or a one-zone polar grid refuses to advance in it
    (and the FP64 path still runs them)."""
    import knc
    from knc import workloads
    one_zone = workloads.wind_small()
    one_zone.mesh.num_polar_zones = 1
    for w in (workloads.sphere_small(), one_zone):
        g = knc.build_solver(w)
        g.set_precision(knc.abi.KNC_PRECISION_MIXED)
        with pytest.raises(knc.abi.KncError) as exc:
            g.advance(1)
        assert exc.value.status == knc.abi.KNC_ERR_UNSUPPORTED
        g.set_precision(knc.abi.KNC_PRECISION_FP64)
        g.advance(1)
