"""Ensemble sharding across processes (one GPU each).

Members and variables are independent columns of the stacked leading
dimension (mg_parameter.f90:296-297; S2C_ens, mg_transfer.f90:269-301), and
the filter never mixes them, so a batch splits across ranks by members with
no exchange on the data path.  The only collective is the timing reduction
(max over ranks) that a benchmark takes.
"""
from __future__ import annotations

from typing import Tuple


def member_range(n_members: int, rank: int, world: int) -> Tuple[int, int]:
    """Contiguous [begin, end) members of `rank` out of `world` (sizes differ by at most one)."""
    if world <= 0 or not (0 <= rank < world) or n_members < 0:
        raise ValueError("bad shard request")
    base, extra = divmod(n_members, world)
    begin = rank * base + min(rank, extra)
    return begin, begin + base + (1 if rank < extra else 0)


def max_over_ranks(value: float, device=None) -> float:
    """Maximum of `value` over the default process group (identity without one)."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(value)
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())
