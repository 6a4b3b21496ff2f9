"""Multi-GPU runs are independent replicas: the benchmark's host logic (gloo
barrier, max over ranks of the timed region, rank-0 output) with world_size 2
on the CPU."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world), LOCAL_RANK=str(rank))
    import bench
    r, w, local, pg = bench.dist_setup(world)
    bench.barrier(pg)
    m = bench.max_over_ranks(pg, 10.0 + r)
    q.put((r, w, local, m))
    pg.destroy_process_group()


def test_two_replicas_max_over_ranks():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
    assert [o[0] for o in out] == [0, 1]
    assert all(o[1] == 2 and o[3] == 11.0 for o in out)
