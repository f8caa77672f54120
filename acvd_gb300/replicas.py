"""Replica runs over the GPUs of one node (one process per GPU, as torchrun launches them).

A single mesh does not shard without a halo exchange and a per-step all-reduce of the
cluster accumulators, which the reference has neither of, so a multi-GPU run is N
independent replicas of the same solve: no collective on the data path, only the
timing reduced as the maximum over the ranks.  The helpers take the backend as an
argument so that the same code runs as NCCL ranks on GPUs and as gloo ranks on CPU.
"""
from __future__ import annotations

import os


def world() -> tuple[int, int, int]:
    """(world size, rank, local rank) from the launcher's environment."""
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def init(backend: str = "nccl") -> None:
    """Joins the process group when there is more than one rank."""
    ws, _, _ = world()
    if ws > 1:
        import torch.distributed as dist
        if not dist.is_initialized():
            dist.init_process_group(backend)


def max_over_ranks(value: float, device="cpu") -> float:
    """The largest value over the ranks (the slowest replica's time)."""
    ws, _, _ = world()
    if ws == 1:
        return float(value)
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def barrier() -> None:
    ws, _, _ = world()
    if ws > 1:
        import torch.distributed as dist
        dist.barrier()


def aggregate_rate(units_per_rank: float, ms_max: float) -> float:
    """Whole-job throughput: every rank processed units_per_rank in at most ms_max."""
    ws, _, _ = world()
    return ws * units_per_rank / (ms_max / 1000.0)
