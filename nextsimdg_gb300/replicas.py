"""Work split for runs on several GPUs (one process per GPU).

The dynamics of one grid has no data-parallel split without a halo exchange
per mEVP iteration, so several GPUs run independent replicas or independent
ensemble members: members are sharded across ranks with no collective on the
data path; the only communication is the barrier and the max-reduction of
the timings on the host (gloo).
"""
from __future__ import annotations

import os


def shard(n_members: int, rank: int, world: int) -> range:
    """Contiguous block of member indices owned by `rank` (sizes differ by at most one)."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError("bad rank/world")
    base, extra = divmod(n_members, world)
    lo = rank * base + min(rank, extra)
    return range(lo, lo + base + (1 if rank < extra else 0))


def init_from_env():
    """(world, rank, local_rank); initialises a gloo process group when world > 1."""
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
        if not dist.is_initialized():
            dist.init_process_group("gloo", rank=rank, world_size=world)
    return world, rank, local


def max_over_ranks(x: float, world: int) -> float:
    if world == 1:
        return float(x)
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(x)], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def sum_over_ranks(x: float, world: int) -> float:
    if world == 1:
        return float(x)
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(x)], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())


def barrier(world: int):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def throughput(units_this_rank: float, seconds_this_rank: float, world: int) -> float:
    """Whole-job units per second: all ranks' units over the slowest rank's time."""
    return sum_over_ranks(units_this_rank, world) / max_over_ranks(seconds_this_rank, world)
