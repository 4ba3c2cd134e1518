"""Replica timing across ranks (one independent replica of the apply per GPU).

The apply is not sharded across GPUs in this build: every rank holds the whole
basis and operator and processes its own vectors.  Whole-job throughput is the
sum of the ranks' units over the slowest rank's time.
"""
from __future__ import annotations


def aggregate(units_local: float, ms_local: float, device=None):
    """Returns (total units, max ms over ranks); a barrier precedes the reduction."""
    import torch
    import torch.distributed as dist

    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return units_local, ms_local
    dist.barrier()
    t = torch.tensor([ms_local], dtype=torch.float64, device=device)
    u = torch.tensor([units_local], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    dist.all_reduce(u, op=dist.ReduceOp.SUM)
    return float(u.item()), float(t.item())
