"""Replica-parallel runs over several processes (one GPU each): every rank
advances its own independent system with its own seeds, and the only
exchange is the final reduction of the measurement -- the slowest rank's
time and the sum of the particle-steps.  No collective touches the data
path (the cg-gcmc-bd loop has no exchange step between systems)."""
from __future__ import annotations

SEED_STRIDE = 1000


def replica_seed(base: int, rank: int) -> int:
    """Workload seed of rank `rank`: disjoint positions and noise streams."""
    return base + SEED_STRIDE * rank


def aggregate(t_ms: float, particle_steps: float, device: str = "cpu"):
    """(slowest rank's time in ms, all ranks' particle-steps); identity when
    torch.distributed is not initialised."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()):
        return t_ms, particle_steps
    tm = torch.tensor([t_ms], dtype=torch.float64, device=device)
    ps = torch.tensor([particle_steps], dtype=torch.float64, device=device)
    dist.all_reduce(tm, op=dist.ReduceOp.MAX)
    dist.all_reduce(ps, op=dist.ReduceOp.SUM)
    return float(tm[0]), float(ps[0])
