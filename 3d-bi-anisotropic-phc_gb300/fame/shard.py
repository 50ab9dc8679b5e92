"""Host-side sharding of a k-point band path over ranks (one process per GPU).

k-points are independent (band_structure_woodpile_Lanczos_n60_gamma0p2.m:45-93
loops over them), so the path is cut into batches and rank r of N takes
batch (s*N + r) mod B at step s: no data collective, only the timer is
reduced (max over ranks).  Works with any torch.distributed backend (gloo
on CPU tensors, nccl on CUDA tensors).
"""
from __future__ import annotations

import os


def env_rank():
    """(rank, world_size, local_rank) from the launcher's environment."""
    return int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")), \
        int(os.environ.get("LOCAL_RANK", "0"))


def batch_index(step: int, rank: int, world: int, nbatches: int) -> int:
    """Batch solved by `rank` at `step`."""
    return (step * world + rank) % nbatches


def batches_of(rank: int, world: int, steps: int, nbatches: int, first_step: int = 0):
    """Batch indices of `rank` for steps first_step .. first_step+steps-1."""
    return [batch_index(s, rank, world, nbatches) for s in range(first_step, first_step + steps)]


def max_over_ranks(value: float, device="cpu") -> float:
    """Max of a scalar over the default process group (identity without one)."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(value)
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def whole_job_rate(units_per_rank_step: int, steps: int, world: int, t_max: float) -> float:
    """Units processed by all ranks per second of the slowest rank."""
    return units_per_rank_step * steps * world / t_max
