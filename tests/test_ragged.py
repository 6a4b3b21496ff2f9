"""Edge shapes: blocks whose rows are not a multiple of any tile or strip
height (nr = 20) and whose columns are not a multiple of a warp or a strip
(nq = 100), a one-zone polar grid, and an empty block set.

Every launch form must match the CPU oracle bit for bit on the FP64 path and
the other forms bit for bit on the mixed path; partial tiles, partial strips
and partial chunks of the host-state advance all occur here.
"""
import numpy as np
import pytest

from helpers import field_errors, make_pair, zone_relative_errors

pytestmark = pytest.mark.gpu

FORMS = {
    "tile4": dict(tile_rows=4),
    "tile8": dict(tile_rows=8),
    "tile16": dict(tile_rows=16),
    "tma8": dict(tile_rows=8, tma=True),
    "strip8": dict(tile_rows=8, strip=True),
    "strip16": dict(tile_rows=16, strip=True),
    "fused8": dict(tile_rows=8, fused=True),
}


def _ragged(nq=100, nr=20):
    from knc import workloads
    w = workloads.wind_small()
    w.mesh.block_size = nr
    w.mesh.num_polar_zones = nq
    return w


@pytest.mark.parametrize("form", sorted(FORMS))
def test_ragged_fp64_matches_oracle(form):
    w = _ragged()
    g, o = make_pair(w)
    g.set_tuning(**FORMS[form])
    for _ in range(2):
        g.advance(3)
        o.advance(3)
    assert max(zone_relative_errors(g.state(), o.state())) == 0.0
    assert g.time() == o.time()


def test_ragged_mixed_forms_agree():
    import knc
    w = _ragged()
    states = {}
    for form in sorted(FORMS) + ["strip16_deferred"]:
        s = knc.build_solver(w)
        s.set_precision(knc.abi.KNC_PRECISION_MIXED)
        s.set_tuning(**(dict(tile_rows=16, strip=True, deferred=True) if form == "strip16_deferred" else FORMS[form]))
        s.advance(5)
        states[form] = s.state()
    ref = states.pop("tile8")
    for form, st in states.items():
        assert max(zone_relative_errors(st, ref)) == 0.0, form
    f64 = knc.build_solver(w)
    f64.advance(5)
    assert max(field_errors(ref, f64.state(), momentum_scale=True)) < 1e-5


def test_ragged_host_advance():
    import knc
    w = _ragged()
    a, b = knc.build_solver(w), knc.build_solver(w)
    zones = sum(int(np.prod(a.shape_of(i))) for i in a.block_indexes())
    pc, ps = knc.solver.PinnedArray((zones, 4)), knc.solver.PinnedArray((zones,))
    a.get_state(pc.array, ps.array)
    a.advance_host(pc.array, ps.array, 2)
    b.advance(2)
    oc, os_ = np.empty((zones, 4)), np.empty(zones)
    b.get_state(oc, os_)
    assert np.array_equal(pc.array, oc) and np.array_equal(ps.array, os_)


@pytest.mark.parametrize("form", ["tile4", "tile8", "tile16"])
def test_one_polar_zone_fp64(form):
    """num_polar_zones = 1: no polar faces; warp strips are refused there."""
    import knc
    w = _ragged(nq=1, nr=64)
    g, o = make_pair(w)
    with pytest.raises(knc.abi.KncError):
        g.set_tuning(**FORMS["strip8"])
    g.set_tuning(**FORMS[form])
    g.advance(4)
    o.advance(4)
    assert max(zone_relative_errors(g.state(), o.state())) == 0.0
    # the host-state advance takes the whole-copy form here
    zones = sum(int(np.prod(g.shape_of(i))) for i in g.block_indexes())
    pc, ps = knc.solver.PinnedArray((zones, 4)), knc.solver.PinnedArray((zones,))
    g.get_state(pc.array, ps.array)
    g.advance_host(pc.array, ps.array, 2)
    o.advance(2)
    off = 0
    for i, (c, sc) in sorted(o.state().items()):
        n = c.shape[0] * c.shape[1]
        assert np.array_equal(pc.array[off:off + n], c.reshape(-1, 4))
        assert np.array_equal(ps.array[off:off + n], sc.reshape(-1))
        off += n


def test_empty_block_set_rejected():
    import knc
    w = _ragged()
    s = knc.Solver(w.hydro, w.mesh)
    s.set_model(w.model)
    with pytest.raises(knc.abi.KncError):
        s.advance(1)
