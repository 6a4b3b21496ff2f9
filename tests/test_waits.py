"""Bounded device waits, tested without a GPU fault.

Errors are values in the reference (src/traits.rs:78-82); the library keeps
its device waits in that contract. A wait that cannot complete gives up after
a bounded number of polls and the stage reports KNC_ERR_TIMEOUT, with the
input state intact and the context usable after the state is reloaded. The
tests make the waits run out on purpose: a grid barrier of the fused stage
that counts one arrival more than the grid makes, and an mbarrier that
nothing arrives on (the poll loop of the tensor-copy update, with no copy
issued). Both waits are short (a few thousand polls).
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("precision", ["fp64", "mixed", "mixed_deferred", "mixed_deferred_wide"])
def test_fused_barrier_gives_up_and_reports_timeout(precision):
    """mixed_deferred: the fused stage with the deferring recovery (its
    first barrier follows phase A's claimed items); _wide: one 20-warp CTA
    per SM."""
    import knc
    from knc import abi, workloads
    w = workloads.wind_small()
    s = knc.build_solver(w)
    ref = knc.build_solver(w)
    for g in (s, ref):
        if precision != "fp64":
            g.set_precision(abi.KNC_PRECISION_MIXED)
        if precision.startswith("mixed_deferred"):
            g.set_tuning(tile_rows=16, fused=True, strip=True, deferred=True,
                         ctas_per_sm=1 if precision.endswith("wide") else 0)
        else:
            g.set_tuning(tile_rows=8, fused=True)
        g.advance(1)
    zones = sum(int(np.prod(s.shape_of(i))) for i in s.block_indexes())
    cons, scal = np.empty((zones, 4)), np.empty(zones)
    s.get_state(cons, scal)
    s.set_wait_test(polls=4096, unreachable=True)
    with pytest.raises(abi.KncError) as exc:
        s.advance(1)
    assert exc.value.status == abi.KNC_ERR_TIMEOUT
    # no stage wrote the state: it is the state before the failed call
    after_c, after_s = np.empty_like(cons), np.empty_like(scal)
    s.get_state(after_c, after_s)
    assert np.array_equal(after_c, cons) and np.array_equal(after_s, scal)
    # the context is usable: reload the state, advance, compare with a solver
    # that never timed out
    s.set_wait_test(0, False)
    s.set_state(cons, scal)
    s.advance(1)
    ref.advance(1)
    a, b = s.state(), ref.state()
    for k in b:
        assert np.array_equal(a[k][0], b[k][0]) and np.array_equal(a[k][1], b[k][1])


def test_copy_wait_gives_up_on_a_barrier_nothing_arrives_on():
    from knc import abi
    lib = abi.load()
    out = C.c_int32(-1)
    assert lib.knc_selftest_copy_wait(2048, C.byref(out)) == abi.KNC_OK
    assert out.value == 1
    # the device is still usable afterwards
    import knc
    from knc import workloads
    g = knc.build_solver(workloads.wind_small())
    g.advance(1)
