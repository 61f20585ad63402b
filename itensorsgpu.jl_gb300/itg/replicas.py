"""Replica parallelism across GPUs: one process per GPU, no collective on the
data path.

A single DMRG sweep does not shard (it is sequential over bonds, and splitting
one matvec across GPUs would all-gather psi every matvec), so N GPUs run
independent work: the same H_eff benchmark per GPU, or disjoint blocks of
independent chains (the many-chain workload).  Ranks meet only on the host,
to take the slowest rank's time and to gather per-instance results in
instance order.  These helpers use torch.distributed when it is initialised
(NCCL on GPUs, gloo on CPU) and are the identity on one process.
"""
from __future__ import annotations


def world_rank():
    """(world size, rank) from torch.distributed, else from the launcher's
    environment, else (1, 0)."""
    import os
    try:
        import torch.distributed as dist
        if dist.is_available() and dist.is_initialized():
            return dist.get_world_size(), dist.get_rank()
    except ImportError:  # pragma: no cover
        pass
    return int(os.environ.get("WORLD_SIZE", "1")), int(os.environ.get("RANK", "0"))


def shard(count: int, world: int, rank: int) -> range:
    """Contiguous block of instance indices owned by `rank`: sizes differ by at
    most one, every index owned exactly once, in rank order."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError(f"rank {rank} outside a world of {world}")
    base, extra = divmod(count, world)
    start = rank * base + min(rank, extra)
    return range(start, start + base + (1 if rank < extra else 0))


def max_over_ranks(value: float, device=None) -> float:
    """The largest `value` over all ranks (the job's time is the slowest rank's)."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(value)
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def gather_in_order(local: list, count: int) -> list:
    """Concatenate every rank's per-instance results (each rank holding its
    `shard`) into one list in instance order; the same list on every rank."""
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return list(local)
    world = dist.get_world_size()
    parts = [None] * world
    dist.all_gather_object(parts, list(local))
    out = [x for p in parts for x in p]
    if len(out) != count:
        raise RuntimeError(f"gathered {len(out)} results for {count} instances")
    return out
