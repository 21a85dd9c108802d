"""Replica helpers: one process per GPU, independent work units, no data-path collective.

Templates, coefficient vectors, HMC chains and galaxies are independent, so N GPUs run N
replicas of the same hot path (the reference parallelises the same units over Julia
threads, e.g. hmc_sample.jl:116-139 and generic_fitting.jl:596-599).  The only
cross-rank traffic is host bookkeeping: a barrier around timed regions, the maximum of
the per-rank times and the sum of per-rank counts.  Works with the NCCL backend on GPUs
and with gloo on CPU (the tests).
"""
from __future__ import annotations

import os


def dist_env():
    """(world size, rank, local rank) from the torchrun environment (1, 0, 0 alone)."""
    return (int(os.environ.get("WORLD_SIZE", "1")), int(os.environ.get("RANK", "0")),
            int(os.environ.get("LOCAL_RANK", "0")))


def _device_for_backend():
    import torch
    import torch.distributed as dist
    if dist.get_backend() == "nccl":
        return torch.device("cuda", torch.cuda.current_device())
    return torch.device("cpu")


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def max_over_ranks(world, x: float) -> float:
    """Maximum of a per-rank value (the slowest rank's time bounds the job)."""
    if world == 1:
        return float(x)
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(x)], dtype=torch.float64, device=_device_for_backend())
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def sum_over_ranks(world, x: float) -> float:
    """Sum of a per-rank count (units processed by the whole job)."""
    if world == 1:
        return float(x)
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(x)], dtype=torch.float64, device=_device_for_backend())
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())


def shard(n_units: int, world: int, rank: int) -> range:
    """Contiguous block of independent units for this rank; blocks differ in size by at
    most one and cover [0, n_units) exactly once."""
    if world < 1 or not (0 <= rank < world) or n_units < 0:
        raise ValueError("invalid world / rank / unit count")
    base, extra = divmod(n_units, world)
    start = rank * base + min(rank, extra)
    return range(start, start + base + (1 if rank < extra else 0))
