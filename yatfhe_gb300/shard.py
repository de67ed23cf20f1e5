"""Sharding of independent bootstraps over ranks (one process per GPU).

Every bootstrap is independent and only reads its key, so a multi-GPU job splits its
ciphertexts (or tenants) across ranks with no collective on the data path; the only
collectives are the timing barrier and the max-over-ranks of the measured time.
"""
from __future__ import annotations


def shard_range(count: int, rank: int, world: int) -> tuple[int, int]:
    """[begin, end) of the `count` units that `rank` of `world` processes (contiguous, sizes
    differing by at most one)."""
    if world < 1 or not 0 <= rank < world or count < 0:
        raise ValueError("bad shard request")
    return count * rank // world, count * (rank + 1) // world


def shard_tenants(tenant_ids, rank: int, world: int) -> list:
    """Tenants owned by `rank` (round robin, so a tenant's key lives on one GPU only)."""
    return [t for i, t in enumerate(tenant_ids) if i % world == rank]


def max_over_ranks(value: float, device=None) -> float:
    """Maximum of `value` over all ranks of the default process group (identity when the
    job is a single process)."""
    import torch
    import torch.distributed as dist

    if not dist.is_available() or not dist.is_initialized() or dist.get_world_size() == 1:
        return float(value)
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())
