"""Multi-process helpers: one process per GPU, independent work per rank.

A single CNF instance does not shard (every pass reads the whole clause
database), so N GPUs run N replicas or disjoint shares of many instances;
the only cross-rank steps are the timing barrier and the max/sum reductions
of the benchmark, never a collective on the data path.
"""
from typing import Sequence


def shard_range(n_items: int, rank: int, world: int) -> range:
    """Contiguous, balanced share of `n_items` for `rank` (sizes differ by <= 1)."""
    if world <= 0 or not 0 <= rank < world:
        raise ValueError("bad rank/world")
    base, extra = divmod(n_items, world)
    start = rank * base + min(rank, extra)
    return range(start, start + base + (1 if rank < extra else 0))


def shard(items: Sequence, rank: int, world: int) -> list:
    return [items[i] for i in shard_range(len(items), rank, world)]


def _reduce(x: float, op: str, device=None) -> float:
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()):
        return x
    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX if op == "max" else dist.ReduceOp.SUM)
    return float(t.item())


def allreduce_max(x: float, device=None) -> float:
    return _reduce(x, "max", device)


def allreduce_sum(x: float, device=None) -> float:
    return _reduce(x, "sum", device)
