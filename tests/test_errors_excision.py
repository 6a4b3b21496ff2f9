"""Hydro failures reported like the reference's HydroError, and the moving
excision surfaces retiring / activating blocks (src/scheme.rs:179-206)."""
import numpy as np
import pytest

from helpers import field_errors, make_pair

pytestmark = pytest.mark.gpu


def _poisoned_pair(field, value, block=2, i=5, j=7):
    import knc
    from knc import workloads
    w = workloads.wind_small()
    _, o = make_pair(w, gpu=False)
    st = o.state()
    cons, scal = st[block]
    cons = cons.copy()
    cons[i, j, field] = value
    o.add_block(block, cons, scal)
    g = knc.Solver(w.hydro, w.mesh)
    g.set_model(w.model)
    for k, (c, s) in o.state().items():
        g.add_block(k, c, s)
    return g, o


@pytest.mark.parametrize("field,value,kind", [(0, -1.0, "NegativeDensity"), (3, -1e-3, "NegativeEnergyDensity")])
def test_failure_reported_at_same_zone(field, value, kind):
    import knc
    g, o = _poisoned_pair(field, value)
    st_o = o.try_advance(1)
    assert st_o == 5   # KNC_ERR_HYDRO
    eo = o.last_error()
    with pytest.raises(knc.HydroError) as exc:
        g.advance(1)
    e = exc.value.error
    assert e["kind"] == kind
    assert (e["block"], e["i"], e["j"]) == (eo.block, eo.i, eo.j) == (2, 5, 7)
    assert e["r"] == eo.r and e["theta"] == eo.theta
    assert e["value"] == pytest.approx(eo.value, rel=1e-12)
    # the context refuses to continue from an invalid state, and recovers on reload
    with pytest.raises(knc.HydroError):
        g.advance(1)


def test_context_usable_after_failure():
    from knc import workloads
    g, o = _poisoned_pair(0, -1.0)
    with pytest.raises(Exception):
        g.advance(1)
    w = workloads.wind_small()
    g.init_from_model(0.0)
    g.advance(1)   # a clean state advances again


def test_moving_excision_matches_oracle():
    from knc import workloads
    w = workloads.wind_small()
    w.mesh.inner_excision_speed = 1.0e12
    w.mesh.outer_excision_speed = 1.0e12
    g, o = make_pair(w)
    seen = set()
    for _ in range(6):
        g.advance(3)
        o.advance(3)
        assert g.block_indexes() == o.block_indexes()
        seen.add(tuple(o.block_indexes()))
        assert g.time() == o.time()
    assert len(seen) > 2   # blocks were retired and activated
    errs = field_errors(g.state(), o.state())
    assert max(errs) <= 1e-12, errs
