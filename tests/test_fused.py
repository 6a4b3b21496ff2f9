"""Launch shapes of a stage: update tile rows, the fused persistent stage and
the autotuner.

Every shape runs the same per-zone and per-face arithmetic in the same order
(a face on a tile edge is solved by both tiles from identical inputs), so all
shapes must give bit-identical states: the FP64 ones equal to the oracle, the
mixed ones equal to each other.
"""
import numpy as np
import pytest

from helpers import make_pair, zone_relative_errors

pytestmark = pytest.mark.gpu

SHAPES = [(4, False), (8, False), (16, False), (4, True), (8, True), (16, True)]
STRIPS = [4, 8, 16, 64]


def _same(a, b):
    return max(zone_relative_errors(a, b)) == 0.0


@pytest.mark.parametrize("tile_rows,fused", SHAPES)
def test_fp64_shapes_match_oracle(tile_rows, fused):
    from knc import workloads
    w = workloads.wind_small()
    g, o = make_pair(w)
    g.set_tuning(tile_rows=tile_rows, fused=fused)
    for _ in range(2):
        g.advance(2)
        o.advance(2)
    assert _same(g.state(), o.state())


@pytest.mark.parametrize("tile_rows,fused", SHAPES)
def test_fp64_uneven_moving_shapes_match_oracle(tile_rows, fused):
    from knc import workloads
    w = workloads.uneven_small(order="RK3")
    g, o = make_pair(w)
    g.set_tuning(tile_rows=tile_rows, fused=fused)
    g.set_batched(True)
    for _ in range(2):
        g.advance(5)
        o.advance(5)
    assert g.block_indexes() == o.block_indexes()
    assert _same(g.state(), o.state())


def _mixed(w, tile_rows, fused, batched, mlp=None, steps=6):
    import knc
    g, _ = make_pair(w, gpu=True)
    g.set_precision(knc.abi.KNC_PRECISION_MIXED)
    if mlp is not None:
        g.set_c2p_guess(knc.abi.KNC_GUESS_MLP, mlp)
    g.set_tuning(tile_rows=tile_rows, fused=fused)
    g.set_batched(batched)
    for _ in range(steps // 3):
        g.advance(3)
    return g


@pytest.mark.parametrize("tile_rows", [4, 8, 16])
def test_mixed_fused_matches_separate(tile_rows):
    from knc import workloads
    w = workloads.wind_small()
    ref = _mixed(w, 8, False, False)
    g = _mixed(w, tile_rows, True, True)
    assert _same(g.state(), ref.state())


def test_mixed_learned_fused_matches_separate():
    from knc import learned, workloads
    wts = learned.init_weights(seed=3)
    wts[-6:-3] = 0.0          # input mean
    wts[-3:] = 1.0            # input scale
    w = workloads.jet_small()
    ref = _mixed(w, 8, False, False, mlp=wts)
    g = _mixed(w, 8, True, True, mlp=wts)
    assert _same(g.state(), ref.state())


def test_mixed_uneven_moving_fused_graph():
    from knc import workloads
    w = workloads.uneven_small(order="RK3")
    ref = _mixed(w, 8, False, False, steps=12)
    g = _mixed(w, 16, True, True, steps=12)
    assert g.block_indexes() == ref.block_indexes()
    assert g.block_indexes()[0] > 0
    assert _same(g.state(), ref.state())


def test_autotune_keeps_state_and_results():
    import knc
    from knc import workloads
    w = workloads.uneven_small()
    g, o = make_pair(w)
    g.set_precision(knc.abi.KNC_PRECISION_FP64)
    before = g.state()
    best, ms = g.autotune(reps=2)
    assert best["tile_rows"] in (4, 8, 16) and ms > 0.0
    assert g.tuning() == best
    assert _same(g.state(), before)
    g.advance(4)
    o.advance(4)
    assert _same(g.state(), o.state())
    assert g.time() == o.time()


def test_tuning_validation():
    import knc
    from knc import workloads
    g, _ = make_pair(workloads.wind_small(), gpu=True)
    with pytest.raises(knc.abi.KncError):
        g.set_tuning(tile_rows=12)
    with pytest.raises(knc.abi.KncError):
        g.set_tuning(tile_rows=8, ctas_per_sm=-1)
    with pytest.raises(knc.abi.KncError):
        g.set_tuning(tile_rows=32)            # tiles: 4, 8 or 16 rows
    with pytest.raises(knc.abi.KncError):
        g.set_tuning(tile_rows=128, strip=True)
    g.set_tuning(tile_rows=32, strip=True)
    assert g.tuning()["strip"]


def test_fused_counts_one_launch_per_stage():
    import ctypes as C
    from knc import workloads
    w = workloads.wind_small()
    g, _ = make_pair(w, gpu=True)
    g.set_tuning(tile_rows=8, fused=True)
    n0 = C.c_int64()
    g.lib.knc_launch_count(g.h, C.byref(n0))
    g.advance(3)
    n1 = C.c_int64()
    g.lib.knc_launch_count(g.h, C.byref(n1))
    assert n1.value - n0.value == 3 * 2      # RK2: two stages per step, one launch each


def test_launch_count_counts_every_kernel():
    """Launches per stage as counted by knc_launch_count: ghost rows,
    recovery, update; the deferring recovery adds its dense FP64 pass."""
    import knc
    from knc import workloads
    w = workloads.wind_small()
    g, _ = make_pair(w, gpu=True)
    g.set_precision(knc.abi.KNC_PRECISION_MIXED)
    for deferred, per_stage in ((False, 3), (True, 4)):
        g.set_tuning(tile_rows=8, strip=True, deferred=deferred)
        n0 = g.launch_count()
        g.advance(2)
        assert g.launch_count() - n0 == 2 * 2 * per_stage


@pytest.mark.parametrize("tile_rows", [4, 8, 16])
def test_mixed_tma_staging_matches(tile_rows):
    """The tensor-copy staged update reads the same values from shared
    memory that the plain update reads from global memory."""
    from knc import workloads
    w = workloads.wind_small()
    ref = _mixed(w, tile_rows, False, False)
    import knc
    g, _ = make_pair(w, gpu=True)
    g.set_precision(knc.abi.KNC_PRECISION_MIXED)
    g.set_tuning(tile_rows=tile_rows, tma=True)
    g.set_batched(True)
    for _ in range(2):
        g.advance(3)
    assert _same(g.state(), ref.state())


def test_mixed_tma_uneven_moving():
    """96 uneven blocks (nq 64..256), moving excision, RK3: tensor-copy staging
    inside the captured fold equals the plain separate launches."""
    import knc
    from knc import workloads
    w = workloads.uneven()
    ref = knc.build_solver(w)
    ref.set_precision(knc.abi.KNC_PRECISION_MIXED)
    g = knc.build_solver(w)
    g.set_precision(knc.abi.KNC_PRECISION_MIXED)
    g.set_tuning(tile_rows=8, tma=True)
    g.set_batched(True)
    for _ in range(2):
        ref.advance(4)
        g.advance(4)
    assert g.block_indexes() == ref.block_indexes()
    assert _same(g.state(), ref.state())


@pytest.mark.parametrize("rows", STRIPS)
def test_fp64_strips_match_oracle(rows):
    from knc import workloads
    w = workloads.wind_small()
    g, o = make_pair(w)
    g.set_tuning(tile_rows=rows, strip=True)
    for _ in range(2):
        g.advance(2)
        o.advance(2)
    assert _same(g.state(), o.state())


def test_fp64_strips_uneven_moving_match_oracle():
    from knc import workloads
    w = workloads.uneven_small(order="RK3", riemann="HLLC")
    g, o = make_pair(w)
    g.set_tuning(tile_rows=16, strip=True)
    g.set_batched(True)
    for _ in range(2):
        g.advance(5)
        o.advance(5)
    assert g.block_indexes() == o.block_indexes()
    assert _same(g.state(), o.state())


@pytest.mark.parametrize("rows", STRIPS)
def test_mixed_strips_match_tiles(rows):
    import knc
    from knc import workloads
    w = workloads.wind_small()
    ref = _mixed(w, 8, False, False)
    g, _ = make_pair(w, gpu=True)
    g.set_precision(knc.abi.KNC_PRECISION_MIXED)
    g.set_tuning(tile_rows=rows, strip=True)
    g.set_batched(True)
    for _ in range(2):
        g.advance(3)
    assert _same(g.state(), ref.state())


def test_mixed_strips_uneven_moving():
    import knc
    from knc import workloads
    w = workloads.uneven()
    ref = knc.build_solver(w)
    ref.set_precision(knc.abi.KNC_PRECISION_MIXED)
    g = knc.build_solver(w)
    g.set_precision(knc.abi.KNC_PRECISION_MIXED)
    g.set_tuning(tile_rows=32, strip=True)
    g.set_batched(True)
    for _ in range(2):
        ref.advance(4)
        g.advance(4)
    assert g.block_indexes() == ref.block_indexes()
    assert _same(g.state(), ref.state())


@pytest.mark.parametrize("rows", [8, 32])
def test_fused_strips_match(rows):
    """The fused stage with warp strips in its update phase: FP64 equal to the
    oracle, mixed equal to the separate strip form."""
    import knc
    from knc import workloads
    w = workloads.uneven_small(order="RK3")
    g, o = make_pair(w)
    g.set_tuning(tile_rows=rows, strip=True, fused=True)
    g.set_batched(True)
    for _ in range(2):
        g.advance(5)
        o.advance(5)
    assert _same(g.state(), o.state())
    w = workloads.wind_small()
    ref = _mixed(w, 8, False, False)
    m, _ = make_pair(w, gpu=True)
    m.set_precision(knc.abi.KNC_PRECISION_MIXED)
    m.set_tuning(tile_rows=rows, strip=True, fused=True)
    m.set_batched(True)
    for _ in range(2):
        m.advance(3)
    assert _same(m.state(), ref.state())


@pytest.mark.parametrize("learned", [False, True])
def test_mixed_deferred_recovery_matches_inline(learned):
    """Zones that need the FP64 recovery, listed and recovered on full warps by
    a second launch, give the bits of the in-place recovery (the W = 100 jet
    has such zones in its nozzle)."""
    import knc
    from knc import learned as L, workloads
    wts = None
    if learned:
        wts = L.init_weights(seed=3)
        wts[-6:-3] = 0.0
        wts[-3:] = 1.0
    w = workloads.jet_small()
    runs = []
    for deferred in (False, True):
        g, _ = make_pair(w, gpu=True)
        g.set_precision(knc.abi.KNC_PRECISION_MIXED)
        if wts is not None:
            g.set_c2p_guess(knc.abi.KNC_GUESS_MLP, wts)
        g.set_tuning(tile_rows=8, strip=True, deferred=deferred)
        g.reset_c2p_stats()
        g.advance(6)
        runs.append(g)
    assert runs[1].c2p_stats()["iters_fp64"] > 0
    assert runs[0].c2p_stats() == runs[1].c2p_stats()
    assert _same(runs[0].state(), runs[1].state())


def _mixed_strips(w, fused, deferred, batched, mlp=None, steps=6, rows=16, ctas=0):
    import knc
    g, _ = make_pair(w, gpu=True)
    g.set_precision(knc.abi.KNC_PRECISION_MIXED)
    if mlp is not None:
        g.set_c2p_guess(knc.abi.KNC_GUESS_MLP, mlp)
    g.set_tuning(tile_rows=rows, strip=True, fused=fused, deferred=deferred, ctas_per_sm=ctas)
    g.set_batched(batched)
    for _ in range(steps // 3):
        g.advance(3)
    return g


@pytest.mark.parametrize("ctas", [0, 1, 5])
@pytest.mark.parametrize("name", ["uneven_small", "jet_small", "wind_small"])
def test_mixed_fused_deferred_matches_separate(name, ctas):
    """The fused stage with the deferring recovery (ghost rows, recovery,
    dense FP64 pass, remaps and update in one cooperative launch) equals the
    separate deferring launches bit for bit: on a moving uneven mesh (remaps
    every stage), on the W = 100 jet with the learned guess (listed zones, so
    the dense pass and its barrier run) and on the wind (neither); with
    4-warp CTAs at 4 (ctas 0) or 5 per SM, and with one 20-warp CTA per SM."""
    from knc import learned, workloads
    w = workloads.WORKLOADS[name]()
    wts = None
    if name == "jet_small":
        wts = learned.init_weights(seed=3)
        wts[-6:-3] = 0.0
        wts[-3:] = 1.0
    steps = 12 if name == "uneven_small" else 6
    ref = _mixed_strips(w, False, True, False, mlp=wts, steps=steps)
    g = _mixed_strips(w, True, True, True, mlp=wts, steps=steps, ctas=ctas)
    assert g.block_indexes() == ref.block_indexes()
    assert _same(g.state(), ref.state())
    assert g.time() == ref.time()


def test_fused_deferred_one_launch_per_stage():
    import knc
    from knc import workloads
    w = workloads.uneven_small(order="RK3")
    g, _ = make_pair(w, gpu=True)
    g.set_precision(knc.abi.KNC_PRECISION_MIXED)
    g.set_tuning(tile_rows=16, strip=True, fused=True, deferred=True)
    # RK3: three stages per step, one launch each; an advance call may add
    # one time-step pass
    n0 = g.launch_count()
    g.advance(4)
    assert g.launch_count() - n0 in (4 * 3, 4 * 3 + 1)

