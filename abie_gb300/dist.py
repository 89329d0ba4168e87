"""Multi-GPU helpers: one process per GPU, no data-path collective.

The gravity hot path shards without communication: independent systems of
an ensemble go to different ranks (each rank draws its own systems, so the
work per GPU stays fixed as GPUs are added: weak scaling), and a large
single-system force or integration runs as one replica per GPU.  The only
collective is the timing reduction: the slowest rank's time and the sum
of the units processed.
"""
import os


def rank_info():
    return (int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")),
            int(os.environ.get("LOCAL_RANK", "0")))


def shard(n, rank, world):
    """Contiguous share [lo, hi) of n items for this rank (sizes differ by at most 1)."""
    lo = n * rank // world
    hi = n * (rank + 1) // world
    return lo, hi


def ensemble_seed0(base, rank, systems_per_rank):
    """First seed of this rank's systems: ranks draw disjoint systems."""
    return base + rank * systems_per_rank


def reduce_timing(seconds, units, device=None):
    """(max seconds over ranks, total units over ranks); identity when not distributed."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()):
        return float(seconds), float(units)
    t = torch.tensor([float(seconds)], dtype=torch.float64, device=device)
    u = torch.tensor([float(units)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    dist.all_reduce(u, op=dist.ReduceOp.SUM)
    return float(t.item()), float(u.item())
