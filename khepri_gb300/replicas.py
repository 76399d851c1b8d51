"""Replica parallelism for sweeps: independent problems split across ranks, no collective on the
data path (the reference scales sweeps with process pools over independent points,
examples/crystal_api/twisted_phc.py:90).  Only timing and result gathering talk across ranks.
"""
from __future__ import annotations

import numpy as np


def chunk_indices(total, batch, step, rank, world):
    """Problem indices solved by `rank` at `step`: successive chunks of `batch` problems, ranks
    interleaved so that every (step, rank) pair gets a distinct chunk; wraps around `total`."""
    start = ((step * world + rank) * batch) % total
    return np.arange(start, start + batch) % total


def max_over_ranks(value, device="cpu"):
    """Largest value of a float over all ranks (the slowest replica sets the job time)."""
    import torch
    import torch.distributed as dist

    if not dist.is_available() or not dist.is_initialized() or dist.get_world_size() == 1:
        return float(value)
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def gather_results(local, device="cpu"):
    """Concatenate per-rank result arrays (equal lengths) on every rank, rank order."""
    import torch
    import torch.distributed as dist

    arr = torch.as_tensor(np.ascontiguousarray(local), device=device)
    if not dist.is_available() or not dist.is_initialized() or dist.get_world_size() == 1:
        return arr.cpu().numpy()
    out = [torch.empty_like(arr) for _ in range(dist.get_world_size())]
    dist.all_gather(out, arr)
    return torch.cat(out).cpu().numpy()
