"""Independent replicas on several GPUs (one process per GPU, launched by torchrun).

The solve path has no exchange step that this backend distributes: a rank solves its own
problems (benchmark replicas, training-data solves for the learned preconditioner).  The
only cross-rank operations are the partition of independent work items and the maximum of
the ranks' timings; both work with the gloo (CPU) and nccl backends.
"""
import os

import torch


def rank_world():
    if torch.distributed.is_available() and torch.distributed.is_initialized():
        return torch.distributed.get_rank(), torch.distributed.get_world_size()
    return int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1"))


def shard(items, rank=None, world=None):
    """Contiguous, balanced share of ``items`` for ``rank`` (sizes differ by at most one)."""
    if rank is None or world is None:
        rank, world = rank_world()
    n = len(items)
    lo = rank * n // world
    hi = (rank + 1) * n // world
    return items[lo:hi]


def max_over_ranks(value, device=None):
    """Maximum of a float over all ranks (the benchmark's whole-job time)."""
    if not (torch.distributed.is_available() and torch.distributed.is_initialized()):
        return float(value)
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    return float(t.item())


def sum_over_ranks(value, device=None):
    if not (torch.distributed.is_available() and torch.distributed.is_initialized()):
        return float(value)
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.SUM)
    return float(t.item())
