"""Multi-GPU layout of the per-cell path: cells are independent, so ranks take contiguous cell ranges
and never exchange data; the only collectives are host-side reductions of timings and statistics."""
from __future__ import annotations


def cell_range(n: int, world: int, rank: int):
    """[lo, hi) of the cells rank ``rank`` of ``world`` owns: contiguous, sizes differing by at most one."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError("bad rank/world")
    return n * rank // world, n * (rank + 1) // world


def reduce_max(value: float, device=None) -> float:
    """Max over ranks of a scalar (identity without an initialised process group)."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return value
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def reduce_sum(value: float, device=None) -> float:
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return value
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())
