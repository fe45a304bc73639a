"""Host logic of running N replicas of the transform path, one per GPU.

The GLQ transforms shard over independent batch items with no exchange step,
so N > 1 means N independent replicas: rank r transforms its own batch (seeds
disjoint from every other rank's), all ranks start the timed region together
(barrier), and the job's time is the maximum over ranks.  There is no
collective on the data path; the only collectives are the barrier and the
max-reduction of the timings."""
from __future__ import annotations


def replica_seed0(rank: int, batch: int) -> int:
    """First seed of rank `rank`'s batch: ranks draw seeds 1.. in disjoint blocks."""
    return 1 + rank * batch


def max_over_ranks(value: float, dist=None, device: str = "cpu") -> float:
    """The maximum of `value` over all ranks (the value itself without a process group)."""
    if dist is None:
        return float(value)
    import torch
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def whole_job_rate(units_per_rank: float, world: int, seconds: float) -> float:
    """Units processed by all ranks per second of the slowest rank."""
    return world * units_per_rank / seconds
