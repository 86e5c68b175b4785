"""Independent replicas on several GPUs (one process per GPU).

A correlation job needs no exchange between GPUs: the whole job fits one
GB300.  Several GPUs therefore run independent replicas -- the same workload
per rank, or a round-robin share of many independent stacks -- and the only
collective is the barrier and the maximum of the per-rank step times used to
report a whole-job rate.  The helpers work on any ``torch.distributed``
backend (NCCL on GPUs, gloo on the CPU for tests).
"""
from __future__ import annotations

import os


def rank_info():
    """(rank, world_size, local_rank) from the torchrun environment."""
    return (int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")),
            int(os.environ.get("LOCAL_RANK", "0")))


def max_over_ranks(x, dist=None, device=None):
    """The maximum of a per-rank float over all ranks (x itself without a
    process group)."""
    if dist is None or not dist.is_initialized():
        return float(x)
    import torch
    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def whole_job_rate(units_per_rank, ms_per_rank, world):
    """Units per second of the whole job when every rank processes
    ``units_per_rank`` units and the slowest takes ``ms_per_rank`` ms."""
    return world * float(units_per_rank) / (float(ms_per_rank) / 1e3)


def shard(items, rank, world):
    """Round-robin share of independent items for one rank: every item goes
    to exactly one rank and the shares differ in size by at most one."""
    return list(items)[rank::world]
