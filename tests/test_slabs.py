"""Radial-slab decomposition (knc.slabs): ranks advance overlapping slabs with
the minimum time step over the slabs and exchange their edge blocks with
their neighbours once per fold; every owned block must equal the
single-domain run bit for bit, and each rank sends only its overlap blocks.

The CPU tests run the oracle as each rank's engine on gloo ranks
(world_size 2); the GPU test runs two library contexts on one GPU in one
process, exchanging through host arrays."""
import os
import socket

import numpy as np
import pytest

from helpers import zone_relative_errors

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _oracle(w):
    import knc_oracle
    o = knc_oracle.Oracle(w.hydro, w.mesh, threads=2)
    o.set_model(w.model)
    o.init_from_model(0.0)
    return o


def _workload(name):
    from knc import workloads
    return {"wind": workloads.wind_small, "sphere": workloads.sphere_small}[name]()


def _rank(rank, world, port, name, folds, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    from knc import slabs
    w = _workload(name)
    eng = _oracle(w)
    all_idx = eng.block_indexes()
    owned = slabs.partition(all_idx, world)[rank]
    dom = slabs.SlabDomain(eng, owned, all_idx, overlap=1, order=int(w.hydro.runge_kutta_order[-1]))

    def allreduce_min(x):
        t = torch.tensor([x], dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.MIN)
        return float(t.item())

    exchange = slabs.torch_neighbour_exchange(dist, rank, world)
    for f in folds:
        slabs.advance_slabs([dom], f, allreduce_min, exchange)
    q.put((rank, {i: (c.copy(), s.copy()) for i, (c, s) in dom.owned_blocks().items()}, eng.time(),
           dom.bytes_sent, len(dom.to_below()) * (rank > 0) + len(dom.to_above()) * (rank < world - 1)))
    dist.destroy_process_group()


@pytest.mark.parametrize("name,world", [("wind", 2), ("sphere", 2), ("wind", 3)])
def test_cpu_ranks_match_single_domain(name, world):
    folds = [6, 5]
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, world, port, name, folds, q)) for r in range(world)]
    for p in procs:
        p.start()
    out = [q.get(timeout=300) for _ in procs]
    for p in procs:
        p.join(timeout=60)
    ref = _oracle(_workload(name))
    for f in folds:
        ref.advance(f)
    merged = {}
    block_bytes = ref.nr * ref.nq * 5 * 8
    for _, blocks, t, sent, edge_blocks in out:
        merged.update(blocks)
        assert t == ref.time()
        # each fold a rank sends its edge blocks to its neighbours, nothing else
        assert sent == len(folds) * edge_blocks * block_bytes
    assert sorted(merged) == ref.block_indexes()
    assert max(zone_relative_errors(merged, ref.state())) == 0.0


def test_partition_and_fold_limit():
    from knc import slabs
    assert slabs.partition(range(10), 3) == [[0, 1, 2, 3], [4, 5, 6], [7, 8, 9]]
    w = _workload("wind")
    eng = _oracle(w)
    dom = slabs.SlabDomain(eng, [0, 1], eng.block_indexes(), overlap=1, order=2)
    assert eng.block_indexes() == [0, 1, 2]
    assert dom.max_fold() == 64 // 4 - 1
    with pytest.raises(ValueError):
        slabs.advance_slabs([dom], dom.max_fold() + 1)


@pytest.mark.gpu
def test_two_gpu_contexts_match_single_domain():
    import knc
    from knc import slabs, workloads
    w = workloads.wind_small()
    ref = knc.build_solver(w)
    ref.set_precision(knc.abi.KNC_PRECISION_FP64)
    all_idx = ref.block_indexes()
    parts = slabs.partition(all_idx, 2)
    doms = [slabs.SlabDomain(knc.build_solver(w), p, all_idx, overlap=1, order=2) for p in parts]
    for f in (8, 7):
        slabs.advance_slabs(doms, f)
        ref.advance(f)
    merged = {}
    for d in doms:
        merged.update(d.owned_blocks())
        assert d.engine.time() == ref.time()
    assert max(zone_relative_errors(merged, ref.state())) == 0.0
