"""Multi-GPU as replicas: pages are independent and the encode path has no
exchange step, so N GPUs run N independent engines on disjoint shares of the
pages and only the timing is combined (the slowest rank sets the job time).
No collective touches the data path."""
from __future__ import annotations

from typing import List, Sequence, TypeVar

T = TypeVar("T")


def shard(items: Sequence[T], rank: int, world: int) -> List[T]:
    """The pages rank `rank` of `world` encodes: every world-th page from
    `rank` on, so shares differ by at most one page."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError(f"rank {rank} outside a world of {world}")
    return list(items[rank::world])


def max_over_ranks(value: float, device=None) -> float:
    """The largest `value` over the ranks of the default process group (the
    value itself without one). Works with the gloo and nccl backends."""
    import torch
    import torch.distributed as td

    if not (td.is_available() and td.is_initialized()):
        return float(value)
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    td.all_reduce(t, op=td.ReduceOp.MAX)
    return float(t.item())


def whole_job_rate(units_per_rank: float, world: int, job_seconds: float) -> float:
    """Throughput of the whole job: all ranks' units over the slowest rank's
    time."""
    return world * units_per_rank / job_seconds
