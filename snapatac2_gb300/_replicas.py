"""Throughput of independent replicas, one process per GPU.

The embedding path does not shard across GPUs here (one dataset per GPU,
no collective in the data path); a run on N GPUs is N replicas.  The
whole-job figure is the units all ranks processed over the slowest rank's
time, which is what this helper reduces (SUM of units, MAX of time) over
the default process group.  With no process group, or one rank, it returns
its inputs.
"""
from __future__ import annotations

import torch


def replica_throughput(units: float, ms: float, device=None) -> tuple[float, float]:
    """(total units over ranks, maximum milliseconds over ranks)."""
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(units), float(ms)
    u = torch.tensor([float(units)], dtype=torch.float64, device=device)
    m = torch.tensor([float(ms)], dtype=torch.float64, device=device)
    dist.all_reduce(u, op=dist.ReduceOp.SUM)
    dist.all_reduce(m, op=dist.ReduceOp.MAX)
    return float(u.item()), float(m.item())
