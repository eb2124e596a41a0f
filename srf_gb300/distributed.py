"""Event-sharded list-mode OSEM over several processes, one GPU each.

The reference distributes a reconstruction by events: each worker takes a contiguous share of the
list-mode events (srfnef/func_classes/distribute.py:60-71) and a master sums the workers' partial
results (srfnef/mixin/master_mixin.py:59-67). Here every rank holds the whole image x and the
sensitivity image. Each subset's events are split into one contiguous shard per rank (sizes
differ by at most one event; nothing is dropped). Every subset step then runs as follows:

1. each rank runs the fused subset step (projection, ratio, backprojection) on its shard, into
   its two backprojection accumulators (one flat buffer);
2. one all-reduce (sum) of that buffer over the ranks;
3. every rank applies the identical multiplicative update x <- x * bp / emap.

The result is the single-process OSEM's, up to the order of the floating-point sums. Nothing but
the collective moves data between ranks, and remote data reaches a rank only through it.

The orchestration is independent of what computes a subset step: an *engine* is any object with
``subset(lors, y, **kw)``, ``accumulators() -> torch.Tensor`` (the flat sum buffer) and
``update(emap, guard_zero)``. On GPUs it is ``kernels.SubsetState`` (NCCL all-reduce).
"""
from __future__ import annotations

from typing import List, Optional, Sequence, Tuple

import torch


def shard_range(n: int, rank: int, world: int) -> Tuple[int, int]:
    """[lo, hi) of rank's contiguous shard of n items; the first n % world ranks get one more."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError(f"rank {rank} outside a world of {world}")
    if n < 0:
        raise ValueError("negative item count")
    base, extra = divmod(n, world)
    lo = rank * base + min(rank, extra)
    return lo, lo + base + (1 if rank < extra else 0)


def subset_shards(n: int, n_sub: int, rank: int, world: int) -> List[Tuple[int, int]]:
    """Global [lo, hi) event ranges of rank's shard of each of the n_sub subsets. Subset k holds
    events [k * n_per, (k + 1) * n_per) of the subset-ordered list, n_per = n // n_sub (the
    remainder is left out, as the single-process OSEM does)."""
    if n_sub < 1:
        raise ValueError("n_sub must be >= 1")
    n_per = n // n_sub
    out = []
    for k in range(n_sub):
        a, b = shard_range(n_per, rank, world)
        out.append((k * n_per + a, k * n_per + b))
    return out


def world_of(group=None) -> Tuple[int, int]:
    """(rank, world size) of the process group, (0, 1) without an initialised group."""
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()):
        return 0, 1
    return dist.get_rank(group), dist.get_world_size(group)


class ShardedOsem:
    """Runs subset steps of an event-sharded OSEM on one rank.

    ``step(lors_shard, y_shard, emap)`` is one subset step: the engine's subset pass over this
    rank's shard, the all-reduce of its accumulators, then the update. With one rank the
    all-reduce is skipped and the step equals the engine's own."""

    def __init__(self, engine, group=None):
        self.engine = engine
        self.group = group
        self.rank, self.world = world_of(group)

    def reduce(self) -> None:
        if self.world > 1:
            import torch.distributed as dist
            dist.all_reduce(self.engine.accumulators(), op=dist.ReduceOp.SUM, group=self.group)

    def step(self, lors: torch.Tensor, y: Optional[torch.Tensor], emap, *, guard_zero: bool = True,
             **subset_kw) -> None:
        self.engine.subset(lors, y, **subset_kw)
        self.reduce()
        self.engine.update(emap, guard_zero=guard_zero)

    def iteration(self, shards: Sequence[torch.Tensor], ys: Optional[Sequence[Optional[torch.Tensor]]],
                  emap, *, guard_zero: bool = True, adds=None, **subset_kw) -> None:
        """One pass over all subsets: shards[k] (ys[k], adds[k]) is this rank's part of subset k."""
        for k, lors in enumerate(shards):
            kw = dict(subset_kw)
            if adds is not None:
                kw["add"] = adds[k]
            self.step(lors, None if ys is None else ys[k], emap, guard_zero=guard_zero, **kw)
