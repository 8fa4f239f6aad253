"""Weak-scaling replicas of the chemistry step over the GPUs of one node.

The chemistry step has no exchange between cells (the only vertical coupling,
the column sums of the rate stage, stays inside a column), so several GPUs
run replicas: every rank integrates its own grid, with no data-path
collective. The whole-job figure is the cells of all ranks over the slowest
rank's time, the only collective being that one reduction of a timing.
"""
from __future__ import annotations


def replica_seed(base: int, rank: int) -> int:
    """Seed of rank `rank`'s synthetic grid (different on every rank)."""
    return base + rank


def max_over_ranks(value: float) -> float:
    """The largest `value` over the ranks of the default process group (the
    value itself without one): timings are reported for the slowest rank."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(value)
    device = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def whole_job_rate(cells_per_rank: int, world: int, steps: int, seconds: float) -> float:
    """Cell-steps per second of the whole job: every rank's cells, each step,
    over the time of the slowest rank."""
    return cells_per_rank * world * steps / seconds
