"""Uneven blocks: per-block (nr, nq) with polar-resolution halo remaps.

The reference gives every block Mesh::block_size x num_polar_zones zones
(src/mesh.rs:84-113); per-block shapes are this library's extension for the
batched workload of uneven blocks. The oracle carries the same extension
(oracle/knc_oracle.cpp `halo_value`), so the FP64 GPU path must still match it
to 1e-12 (and is expected to match bit for bit): halo rows from a finer
neighbour are its zones merged conservatively and recovered with the
reference's Newton iteration, from a coarser neighbour copied.
"""
import numpy as np
import pytest

from helpers import field_errors, make_pair, zone_relative_errors

TOL = 1e-12


def _equal_shape_state(w, shapes):
    import knc_oracle
    o = knc_oracle.Oracle(w.hydro, w.mesh, threads=4)
    if shapes:
        n = len(w.mesh.grid_block_indexes(0.0)) + 4
        o.set_block_shapes(0, [w.mesh.block_size] * n, [w.mesh.num_polar_zones] * n)
    o.set_model(w.model)
    o.init_from_model(0.0)
    o.advance(3)
    return o.state()


def test_oracle_equal_shapes_change_nothing():
    from knc import workloads
    w = workloads.wind_small()
    a = _equal_shape_state(w, False)
    b = _equal_shape_state(w, True)
    assert max(zone_relative_errors(a, b)) == 0.0


def test_oracle_rejects_bad_shapes():
    import knc_oracle
    from knc import workloads
    w = workloads.uneven_small()
    o = knc_oracle.Oracle(w.hydro, w.mesh, threads=1)
    with pytest.raises(Exception):
        o.set_block_shapes(0, [32], [48])     # not nq0 * 2^m
    with pytest.raises(Exception):
        o.set_block_shapes(0, [1], [32])      # fewer than 2 radial zones
    o.set_block_shapes(3, [24], [256])
    assert o.shape_of(3) == (24, 256)
    assert o.shape_of(4) == (w.mesh.block_size, w.mesh.num_polar_zones)


def test_oracle_uneven_runs_and_moves():
    import knc_oracle
    from knc import workloads
    w = workloads.uneven_small()
    o = knc_oracle.Oracle(w.hydro, w.mesh, threads=4)
    w.apply_shapes(o)
    o.set_model(w.model)
    o.init_from_model(0.0)
    o.advance(10)
    idx = o.block_indexes()
    assert idx[0] == 1 and idx[-1] == 8      # one block retired, one activated
    for k, (cons, scalar) in o.state().items():
        assert cons.shape == w.shape_of(k) + (4,)
        assert np.isfinite(cons).all() and np.isfinite(scalar).all()
        assert (cons[..., 0] > 0).all()


@pytest.mark.gpu
def test_uneven_fixed_bitwise():
    from knc import workloads
    w = workloads.uneven_small(order="RK2", moving=False)
    g, o = make_pair(w)
    for _ in range(2):
        g.advance(5)
        o.advance(5)
    assert g.block_indexes() == o.block_indexes()
    errs = zone_relative_errors(g.state(), o.state())
    assert max(errs) == 0.0, errs


@pytest.mark.gpu
@pytest.mark.parametrize("riemann", ["HLLE", "HLLC"])
def test_uneven_moving_rk3(riemann):
    from knc import workloads
    w = workloads.uneven_small(order="RK3", riemann=riemann)
    g, o = make_pair(w)
    for _ in range(w.steps // 10):
        g.advance(10)
        o.advance(10)
    assert g.block_indexes() == o.block_indexes()
    assert g.block_indexes()[0] > 0          # the inner excision retired a block
    assert g.time() == o.time()
    errs = field_errors(g.state(), o.state())
    assert max(errs) <= TOL, errs


@pytest.mark.gpu
def test_uneven_graph_matches_stream():
    from knc import workloads
    w = workloads.uneven_small()
    g1, _ = make_pair(w)
    g2, _ = make_pair(w)
    g2.set_batched(True)
    for _ in range(3):
        g1.advance(10)
        g2.advance(10)
    assert max(zone_relative_errors(g1.state(), g2.state())) == 0.0


@pytest.mark.gpu
def test_uneven_mixed_close_to_fp64():
    import knc
    from knc import workloads
    w = workloads.uneven_small()
    g1, _ = make_pair(w, gpu=True)
    g2, _ = make_pair(w, gpu=True)
    g2.set_precision(knc.abi.KNC_PRECISION_MIXED)
    g1.advance(20)
    g2.advance(20)
    assert g1.block_indexes() == g2.block_indexes()
    errs = field_errors(g2.state(), g1.state())
    assert errs[0] <= 1e-5 and errs[3] <= 1e-4, errs


@pytest.mark.gpu
def test_uneven_shape_errors():
    import knc
    from knc import workloads
    w = workloads.uneven_small(moving=False)
    g, _ = make_pair(w, gpu=True)
    nr, nq = w.shape_of(2)
    with pytest.raises(knc.abi.KncError):
        g.set_block_shapes(2, [nr * 2], [nq])       # live block, other shape
    with pytest.raises(knc.abi.KncError):
        g.set_block_shapes(40, [32], [48])          # not nq0 * 2^m
    g.set_block_shapes(2, [nr], [nq])               # same shape is fine
    assert g.shape_of(2) == (nr, nq)
    cons, scalar = g.get_block(2)
    assert cons.shape == (nr, nq, 4) and scalar.shape == (nr, nq)


@pytest.mark.gpu
@pytest.mark.parametrize("learned", [False, True])
def test_uneven_mixed_chained_graph_matches_stream(learned):
    """The mixed stage's chained launches (row-walking recovery, dense FP64
    pass, warp strips) captured per fold with blocks retiring and
    activating: the graph and the direct launches give the same bits."""
    import knc
    from knc import learned as L, workloads
    w = workloads.uneven_small()
    runs = []
    for graph in (False, True):
        g, _ = make_pair(w)
        g.set_precision(knc.abi.KNC_PRECISION_MIXED)
        if learned:
            g.set_c2p_guess(knc.abi.KNC_GUESS_MLP, L.init_weights(seed=5))
        g.set_tuning(tile_rows=16, strip=True, ctas_per_sm=5, deferred=True)
        g.set_batched(graph)
        for _ in range(3):
            g.advance(10)
        runs.append(g)
    assert runs[0].block_indexes() == runs[1].block_indexes()
    assert max(zone_relative_errors(runs[0].state(), runs[1].state())) == 0.0
    assert runs[0].time() == runs[1].time()
