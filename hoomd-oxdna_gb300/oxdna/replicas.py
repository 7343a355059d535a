"""Replica bookkeeping shared by the batched engine and multi-GPU runs.

The force hot path does not shard: a single system is evaluated on one GPU. What
scales across GPUs is independent replicas (each GPU runs its own set, no data-path
collective), so multi-GPU runs only need a deterministic split of replica ids and a
max-over-ranks reduction of timings.
"""

import numpy as np


def shard(n_replicas, rank, world_size):
    """Replica ids owned by ``rank`` (contiguous, sizes differ by at most one)."""
    if world_size < 1 or not 0 <= rank < world_size:
        raise ValueError("bad rank / world size")
    base, extra = divmod(int(n_replicas), int(world_size))
    start = rank * base + min(rank, extra)
    stop = start + base + (1 if rank < extra else 0)
    return np.arange(start, stop)


def max_over_ranks(value, dist=None):
    """Max of a float over the ranks of an initialised torch.distributed group."""
    if dist is None or not dist.is_available() or not dist.is_initialized():
        return float(value)
    import torch
    t = torch.tensor([float(value)], dtype=torch.float64)
    if dist.get_backend() == "nccl":
        t = t.cuda()
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())
