"""Radial-slab decomposition of the block mesh, one domain per rank.

The mesh is split into slabs of whole radial blocks (`partition`). Each rank
advances its slab plus `overlap` blocks of each neighbouring slab as an
independent context; at the cut the context's own ghost block stands in for
the missing neighbour. A stage reads two zones either side (PLM over a
two-zone halo), so after `fold` steps of an order-s Runge-Kutta scheme the
state is exact except within 2 * s * fold zones of a cut: with the overlap at
least that deep, every owned block is bit-identical to a single-domain run.
After each fold a rank sends its first `overlap` owned blocks to the rank
below and its last `overlap` owned blocks to the rank above, and refreshes
its own overlap from theirs: one neighbour exchange per fold, O(overlap)
bytes, instead of one halo exchange per stage (the dependency of
src/scheme.rs:69-77 is a block's two radial neighbours). The time step is the
minimum over the slabs (`knc_advance_dt`), the one reduction per advance the
decomposition needs.

`engine` is anything with the Solver / Oracle surface (add_block, get_block,
remove_block, block_indexes, shape_of, time_step, advance(fold, dt)).
"""
from __future__ import annotations

from typing import Callable, Dict, List, Sequence, Tuple

import numpy as np


def partition(indexes: Sequence[int], parts: int) -> List[List[int]]:
    """Contiguous runs of block indexes, as even as whole blocks allow."""
    idx = sorted(indexes)
    out, start = [], 0
    for p in range(parts):
        n = len(idx) // parts + (1 if p < len(idx) % parts else 0)
        out.append(idx[start:start + n])
        start += n
    return out


class SlabDomain:
    def __init__(self, engine, owned: Sequence[int], all_indexes: Sequence[int], overlap: int,
                 order: int):
        self.engine = engine
        self.owned = list(owned)
        self.overlap = overlap
        self.order = order
        lo, hi = min(owned), max(owned)
        keep = [i for i in all_indexes if lo - overlap <= i <= hi + overlap]
        for i in engine.block_indexes():
            if i not in keep:
                engine.remove_block(i)
        self.local = sorted(engine.block_indexes())
        # the overlap blocks, owned by the rank below and the rank above
        self.below = [i for i in self.local if i < lo]
        self.above = [i for i in self.local if i > hi]
        self.bytes_sent = 0   # exchange bytes this domain sent, all folds

    def max_fold(self) -> int:
        """Longest fold whose cut error stays inside the overlap."""
        cut_blocks = self.below + self.above
        if not cut_blocks:
            return 1 << 30
        depth = min(self.engine.shape_of(i)[0] for i in cut_blocks) * self.overlap
        return max(depth // (2 * self.order) - 1, 0)

    def owned_blocks(self) -> Dict[int, Tuple]:
        return {i: self.engine.get_block(i) for i in self.owned}

    def to_below(self) -> List[int]:
        """Owned blocks the rank below keeps in its overlap."""
        return self.owned[:self.overlap]

    def to_above(self) -> List[int]:
        """Owned blocks the rank above keeps in its overlap."""
        return self.owned[-self.overlap:]

    def refresh(self, blocks: Dict[int, Tuple]):
        """Overwrite the overlap blocks with their owners' states."""
        for i, (cons, scalar) in blocks.items():
            if i in self.local and i not in self.owned:
                self.engine.add_block(i, cons, scalar)


def in_process_exchange(domains: Sequence[SlabDomain]):
    """Neighbour exchange among domains held by one process."""
    owner = {i: d for d in domains for i in d.owned}
    for d in domains:
        got = {}
        for i in d.below + d.above:
            src = owner[i]
            got[i] = src.engine.get_block(i)
            src.bytes_sent += got[i][0].nbytes + got[i][1].nbytes
        d.refresh(got)


def torch_neighbour_exchange(dist, rank: int, world: int):
    """An exchange for one domain per rank over torch.distributed point-to-
    point messages: each overlap block travels from its owner to the one or
    two neighbours that keep it, as one float64 message of cons + scalar."""
    import torch

    def pack(cons, scalar):
        return torch.from_numpy(np.concatenate([cons.ravel(), scalar.ravel()]))

    def exchange(d: SlabDomain):
        reqs, recv = [], {}
        for peer, send_ids, recv_ids in ((rank - 1, d.to_below(), d.below), (rank + 1, d.to_above(), d.above)):
            if peer < 0 or peer >= world:
                continue
            for i in recv_ids:
                nr, nq = d.engine.shape_of(i)
                buf = torch.empty(int(nr * nq * 5), dtype=torch.float64)
                recv[i] = (buf, nr, nq)
                reqs.append(dist.irecv(buf, src=peer, tag=int(i)))
            for i in send_ids:
                msg = pack(*d.engine.get_block(i))
                d.bytes_sent += msg.numel() * 8
                reqs.append(dist.isend(msg, dst=peer, tag=int(i)))
        for r in reqs:
            r.wait()
        got = {}
        for i, (buf, nr, nq) in recv.items():
            a = buf.numpy()
            n = nr * nq
            got[i] = (a[:4 * n].reshape(nr, nq, 4).copy(), a[4 * n:].reshape(nr, nq).copy())
        d.refresh(got)

    return exchange


def advance_slabs(domains: Sequence[SlabDomain], fold: int,
                  allreduce_min: Callable[[float], float] = None,
                  exchange: Callable[[SlabDomain], None] = None):
    """One fold on every local domain: global dt, advance, neighbour exchange.
    With one process holding all domains the defaults suffice; ranks pass
    their collective min and a per-domain exchange (torch_neighbour_exchange)."""
    for d in domains:
        if fold > d.max_fold():
            raise ValueError(f"fold {fold} exceeds what the overlap covers ({d.max_fold()})")
    local_dt = min(d.engine.time_step() for d in domains)
    dt = allreduce_min(local_dt) if allreduce_min else local_dt
    for d in domains:
        d.engine.advance(fold, dt)
    if exchange is None:
        in_process_exchange(domains)
    else:
        for d in domains:
            exchange(d)
    return dt
