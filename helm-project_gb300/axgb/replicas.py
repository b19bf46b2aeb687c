"""Replica runs on several GPUs of one node, one process per GPU.

The regridding path has no exchange step: every rank applies the operator
to its own fields (weak scaling) or to its own share of independent grid
pairs, so ranks meet only at barriers around a timed region and in the
maximum of the per-rank times. Rank, world size and local rank come from
the torchrun environment (RANK, WORLD_SIZE, LOCAL_RANK, MASTER_ADDR/PORT).
"""

from __future__ import annotations

import os


def world_info():
    """(rank, world_size, local_rank) from the launcher's environment."""
    return (int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")),
            int(os.environ.get("LOCAL_RANK", "0")))


def init(backend: str | None = None) -> None:
    """Join the process group when more than one rank runs (NCCL on GPUs,
    gloo otherwise)."""
    import torch
    import torch.distributed as dist
    _, world, _ = world_info()
    if world > 1 and not dist.is_initialized():
        dist.init_process_group(backend or ("nccl" if torch.cuda.is_available() else "gloo"))


def finalize() -> None:
    import torch.distributed as dist
    if dist.is_initialized():
        dist.destroy_process_group()


def barrier() -> None:
    import torch.distributed as dist
    if dist.is_initialized() and dist.get_world_size() > 1:
        dist.barrier()


def max_over_ranks(value: float) -> float:
    """Maximum of a per-rank scalar (a step time) over all ranks."""
    import torch
    import torch.distributed as dist
    if not dist.is_initialized() or dist.get_world_size() == 1:
        return float(value)
    dev = torch.device("cuda", torch.cuda.current_device()) if dist.get_backend() == "nccl" else torch.device("cpu")
    t = torch.tensor([float(value)], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def aggregate_rate(units_per_rank: float, seconds_max: float, world: int) -> float:
    """Whole-job throughput: the units all ranks processed over the slowest rank's time."""
    return world * units_per_rank / seconds_max


def shard(n: int, rank: int, world: int):
    """Contiguous share [begin, end) of n independent units (grid pairs,
    field blocks) for one rank; shares differ in size by at most one."""
    q, r = divmod(n, world)
    begin = rank * q + min(rank, r)
    return begin, begin + q + (1 if rank < r else 0)
