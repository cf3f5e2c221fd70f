"""Multi-GPU runs of this path are replicas: one process per GPU, each with its
own query set against the same base (the path has no exchange step on one
node: a sharded search would merge per-shard top-k lists, whose ids the
kernels already offset by the shard's first row).
These helpers hold the host-side logic of such a run: per-rank inputs, the
slowest rank's time, and the whole-job rate."""
from __future__ import annotations


def query_seed(rank: int, base: int = 2) -> int:
    """Seed of a rank's synthetic query set (rank 0 keeps the 1-GPU seed)."""
    return base + 1000 * rank


def max_over_ranks(value: float, dist=None, device=None) -> float:
    """The largest value over all ranks (timings: the job ends with its slowest
    rank).  dist: torch.distributed (initialised) or None for one process."""
    if dist is None:
        return float(value)
    import torch
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def whole_job_rate(units_per_rank: float, seconds: float, world: int) -> float:
    """Units per second of the whole job when every rank processed
    units_per_rank and the slowest took seconds (weak scaling)."""
    if seconds <= 0:
        raise ValueError("whole_job_rate: non-positive time")
    return world * units_per_rank / seconds
