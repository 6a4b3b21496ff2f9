"""knc_advance_host: scheme::advance (src/scheme.rs:212-240) on a state held
in host memory, the reference's own calling convention (state in, new state
out).

The streamed form (page-locked buffers) uploads the first step's state and
downloads the last step's by chunks of blocks while the stages run; it must
give bitwise the state, time and iteration of knc_set_state + knc_advance +
knc_get_state, for every RK order, both precisions, each update form, folds
of one and several steps, in place and into separate buffers, and with more
blocks than chunks. Pageable buffers and uneven blocks take the whole-copy
form, with the same result.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _solvers(w, precision, tuning=None):
    import knc
    out = []
    for _ in range(2):
        s = knc.build_solver(w)
        s.set_precision(precision)
        if tuning:
            s.set_tuning(**tuning)
        out.append(s)
    return out


def _host_state(s, pinned):
    import knc
    zones = sum(int(np.prod(s.shape_of(i))) for i in s.block_indexes())
    if pinned:
        keep = (knc.solver.PinnedArray((zones, 4)), knc.solver.PinnedArray((zones,)))
        cons, scal = keep[0].array, keep[1].array
    else:
        keep = None
        cons, scal = np.empty((zones, 4)), np.empty(zones)
    s.get_state(cons, scal)
    return keep, cons, scal


def _by_copies(s, cons, scal, fold):
    s.set_state(cons, scal)
    s.advance(fold)
    oc, os_ = np.empty_like(cons), np.empty_like(scal)
    s.get_state(oc, os_)
    return oc, os_


def _check(w, precision, fold, tuning=None, pinned=True, in_place=True):
    a, b = _solvers(w, precision, tuning)
    for s in (a, b):
        s.advance(2)   # a state with structure, the same on both
    keep, cons, scal = _host_state(a, pinned)
    ref_c, ref_s = _by_copies(b, cons.copy(), scal.copy(), fold)
    if in_place:
        a.advance_host(cons, scal, fold)
        out_c, out_s = cons, scal
    else:
        import knc
        in_c, in_s = cons.copy(), scal.copy()
        outs = (knc.solver.PinnedArray(cons.shape), knc.solver.PinnedArray(scal.shape))
        out_c, out_s = outs[0].array, outs[1].array
        a.advance_host(cons, scal, fold, out_c, out_s)
        assert np.array_equal(cons, in_c) and np.array_equal(scal, in_s)   # inputs untouched
    assert np.array_equal(out_c, ref_c)
    assert np.array_equal(out_s, ref_s)
    assert _time_of(a) == _time_of(b)
    # the device keeps the returned state
    st = a.state()
    off = 0
    for i in a.block_indexes():
        n = int(np.prod(a.shape_of(i)))
        assert np.array_equal(st[i][0].reshape(-1, 4), out_c[off:off + n])
        assert np.array_equal(st[i][1].reshape(-1), out_s[off:off + n])
        off += n
    del keep


def _time_of(s):
    import ctypes as C
    t, n, d = C.c_double(), C.c_int64(), C.c_int64()
    s.lib.knc_get_time(s.h, C.byref(t), C.byref(n), C.byref(d))
    return t.value, n.value, d.value


@pytest.mark.parametrize("order", ["RK1", "RK2", "RK3"])
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("fold", [1, 3])
def test_streamed_matches_copies(order, precision, fold):
    import knc
    from knc import workloads
    w = workloads.wind_small()
    w.hydro.runge_kutta_order = order
    prec = knc.abi.KNC_PRECISION_FP64 if precision == "fp64" else knc.abi.KNC_PRECISION_MIXED
    _check(w, prec, fold)


@pytest.mark.parametrize("tuning", [dict(tile_rows=8), dict(tile_rows=8, tma=True),
                                    dict(tile_rows=16, strip=True, deferred=True)])
def test_streamed_many_blocks_per_chunk(tuning):
    """25 blocks of 8 x 32: chunks of one and two blocks."""
    import knc
    from knc import workloads
    w = workloads.wind_small()
    w.mesh.block_size = 8
    w.mesh.num_polar_zones = 32
    assert w.num_blocks > 16
    _check(w, knc.abi.KNC_PRECISION_MIXED, 2, tuning)


@pytest.mark.parametrize("order,block_size", [("RK3", 6), ("RK3", 4), ("RK2", 4), ("RK1", 2)])
def test_streamed_short_blocks(order, block_size):
    """Blocks of exactly the 2S rows a chunk boundary's shadow copies (S
    stages), and RK3 on blocks of 4 rows, too short for shadows, which the
    call advances through whole-state copies instead."""
    import knc
    from knc import workloads
    w = workloads.wind_small()
    w.mesh.block_size = block_size
    w.mesh.num_polar_zones = 32
    w.hydro.runge_kutta_order = order
    _check(w, knc.abi.KNC_PRECISION_MIXED, 2)


def test_streamed_separate_output():
    import knc
    from knc import workloads
    _check(workloads.wind_small(), knc.abi.KNC_PRECISION_MIXED, 1, in_place=False)


def test_whole_copy_forms():
    """Pageable buffers, and uneven blocks (halo remaps)."""
    import knc
    from knc import workloads
    _check(workloads.wind_small(), knc.abi.KNC_PRECISION_FP64, 2, pinned=False)
    _check(workloads.uneven_small(moving=False), knc.abi.KNC_PRECISION_FP64, 2)


@pytest.mark.parametrize("case", ["newtonian", "srhd_adaptive", "host_model"])
def test_whole_copy_forms_of_other_systems(case):
    """Adaptive time steps (Newtonian, SRHD with adaptive_time_step) and a
    host callback model take the whole-copy form; still bitwise the copies."""
    import knc
    from knc import workloads
    if case == "newtonian":
        w = workloads.sphere_small(riemann="HLLC")
    else:
        w = workloads.wind_small()
        if case == "srhd_adaptive":
            w.hydro.adaptive_time_step = True
    prec = knc.abi.KNC_PRECISION_FP64
    if case == "host_model":
        a, b = _solvers(w, prec)
        def wind(r, q, t):   # AnyPrimitive [u_r, u_theta, rho, p], scalar
            return [1.0, 0.0, 1.0 / (r * r), 1e-4 / (r * r)], 0.0
        for s in (a, b):
            s.set_host_model(wind)
            s.advance(2)
        keep, cons, scal = _host_state(a, True)
        ref_c, ref_s = _by_copies(b, cons.copy(), scal.copy(), 2)
        a.advance_host(cons, scal, 2)
        assert np.array_equal(cons, ref_c) and np.array_equal(scal, ref_s)
        del keep
        return
    _check(w, prec, 2)


def test_moving_mesh_rejected():
    """The block set of a moving mesh changes inside the fold, so flat
    whole-state arrays cannot hold the result: the call refuses."""
    import knc
    from knc import workloads
    w = workloads.uneven_small()
    a = knc.build_solver(w)
    keep, cons, scal = _host_state(a, True)
    with pytest.raises(knc.abi.KncError):
        a.advance_host(cons, scal, 1)
    del keep


@pytest.mark.parametrize("pinned", [True, False])
@pytest.mark.parametrize("field,value,kind", [(0, -1.0, "NegativeDensity"), (3, -1e-3, "NegativeEnergyDensity")])
@pytest.mark.parametrize("row", [5, 0, -1])
def test_failure_reported_like_the_copies(pinned, field, value, kind, row):
    """A poisoned zone in the host state fails the host-state advance at the
    zone the oracle reports (stage 0), in the streamed and the whole-copy
    form; the context then refuses to go on until a state is set again. Rows
    0 and nr - 1 of a block at a chunk boundary are also recovered in the
    neighbouring chunk's shadow block: the block's own zone is reported."""
    import knc
    from helpers import make_pair
    from knc import workloads
    w = workloads.wind_small()
    g, o = make_pair(w)
    keep, cons, scal = _host_state(g, pinned)
    nr, nq = g.shape_of(2)
    i = row % nr
    z = 2 * nr * nq + i * nq + 7          # block 2, zone (i, 7)
    cons[z, field] = value
    c2, s2 = o.get_block(2)
    c2 = c2.copy()
    c2[i, 7, field] = value
    o.add_block(2, c2, s2)
    assert o.try_advance(1) == 5
    eo = o.last_error()
    with pytest.raises(knc.HydroError) as exc:
        g.advance_host(cons, scal, 1)
    e = exc.value.error
    assert e["kind"] == kind
    assert (e["block"], e["i"], e["j"]) == (eo.block, eo.i, eo.j) == (2, i, 7)
    assert e["r"] == eo.r and e["theta"] == eo.theta
    with pytest.raises(knc.HydroError):
        g.advance(1)
    g.init_from_model(0.0)
    g.advance(1)
    del keep


@pytest.mark.parametrize("order", ["RK2", "RK3"])
def test_streamed_jet_matches_copies(order):
    """The W = 100 jet in the mixed stage: its FP64 faces (zones above the
    Lorentz-factor split, the jet's ghost rows among them) give the same bits
    through the host-state chunks as through the device state."""
    import knc
    from knc import workloads
    w = workloads.jet_small()
    w.hydro.runge_kutta_order = order
    _check(w, knc.abi.KNC_PRECISION_MIXED, 2, dict(tile_rows=16, strip=True, deferred=True))
