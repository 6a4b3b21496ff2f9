"""Radial-slab decomposition of the block mesh, one domain per rank.

The mesh is split into slabs of whole radial blocks (`partition`). Each rank
advances its slab plus `overlap` blocks of each neighbouring slab as an
independent context; at the cut the context's own ghost block stands in for
the missing neighbour. A stage reads two zones either side (PLM over a
two-zone halo), so after `fold` steps of an order-s Runge-Kutta scheme the
state is exact except within 2 * s * fold zones of a cut: with the overlap at
least that deep, every owned block is bit-identical to a single-domain run.
After each fold the ranks exchange their owned blocks and refresh the
overlaps (one exchange per fold instead of one halo exchange per stage), and
the time step is the minimum over the slabs (`knc_advance_dt`), the one
reduction per advance the decomposition needs.

`engine` is anything with the Solver / Oracle surface (add_block, get_block,
remove_block, block_indexes, shape_of, time_step, advance(fold, dt)).
"""
from __future__ import annotations

from typing import Callable, Dict, List, Sequence, Tuple


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

    def max_fold(self) -> int:
        """Longest fold whose cut error stays inside the overlap."""
        cut_blocks = [i for i in self.local if i not in self.owned]
        if not cut_blocks:
            return 1 << 30
        depth = min(self.engine.shape_of(i)[0] for i in cut_blocks) * self.overlap
        return max(depth // (2 * self.order) - 1, 0)

    def owned_blocks(self) -> Dict[int, Tuple]:
        return {i: self.engine.get_block(i) for i in self.owned}

    def refresh(self, blocks: Dict[int, Tuple]):
        """Overwrite the overlap blocks with their owners' states."""
        for i, (cons, scalar) in blocks.items():
            if i in self.local and i not in self.owned:
                self.engine.add_block(i, cons, scalar)


def advance_slabs(domains: Sequence[SlabDomain], fold: int,
                  allreduce_min: Callable[[float], float] = None,
                  allgather: Callable[[dict], List[dict]] = None):
    """One fold on every local domain: global dt, advance, exchange owned
    blocks. With one process holding all domains the defaults suffice; ranks
    pass their collective min / all-gather."""
    for d in domains:
        if fold > d.max_fold():
            raise ValueError(f"fold {fold} exceeds what the overlap covers ({d.max_fold()})")
    local_dt = min(d.engine.time_step() for d in domains)
    dt = allreduce_min(local_dt) if allreduce_min else local_dt
    for d in domains:
        d.engine.advance(fold, dt)
    mine = {}
    for d in domains:
        mine.update(d.owned_blocks())
    everyone = allgather(mine) if allgather else [mine]
    merged = {}
    for part in everyone:
        merged.update(part)
    for d in domains:
        d.refresh(merged)
    return dt
