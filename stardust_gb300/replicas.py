"""Host-side logic of multi-GPU runs: one process per GPU, each stepping its
own replica (or its own share of a batch of scenes); no data-path
collective.  The only collectives are the barrier around timed regions and
the max over ranks of the elapsed time, on whatever process group is active
(NCCL on GPUs, gloo in the CPU tests)."""
from __future__ import annotations


def shard(n_items: int, rank: int, world: int) -> list[int]:
    """Items (scenes of a batch) of this rank: rank, rank + world, ...  Every
    item goes to exactly one rank and shares differ by at most one item."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError("need 0 <= rank < world")
    return list(range(rank, n_items, world))


def max_over_ranks(value: float, device="cpu") -> float:
    """The largest value over all ranks (the job's elapsed time)."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(value)
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def sum_over_ranks(value: float, device="cpu") -> float:
    """The sum over ranks (units processed by the whole job)."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(value)
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())


def job_rate(units_this_rank: float, seconds_this_rank: float, device="cpu") -> float:
    """Whole-job throughput: all ranks' units over the slowest rank's time."""
    return sum_over_ranks(units_this_rank, device) / max_over_ranks(seconds_this_rank, device)
