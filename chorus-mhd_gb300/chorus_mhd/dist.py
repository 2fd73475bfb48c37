"""Rank helpers for multi-GPU runs.

The path does not shard across GPUs here: every rank holds whole solves (replicas of a
workload, or its share of an ensemble), so the only collectives are a barrier and a
max-reduction of timings -- no data-path exchange.
"""
from __future__ import annotations

import os


def env():
    """(world_size, rank, local_rank) from the torchrun environment."""
    return (int(os.environ.get("WORLD_SIZE", "1")), int(os.environ.get("RANK", "0")),
            int(os.environ.get("LOCAL_RANK", "0")))


def init(backend: str | None = None):
    world, rank, local = env()
    if world > 1:
        import torch.distributed as dist
        if not dist.is_initialized():
            if backend is None:
                import torch
                backend = "nccl" if torch.cuda.is_available() else "gloo"
            dist.init_process_group(backend=backend)
    return world, rank, local


def barrier(world: int):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def max_over_ranks(world: int, x: float) -> float:
    if world == 1:
        return x
    import torch
    import torch.distributed as dist
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([x], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def sum_over_ranks(world: int, x: float) -> float:
    if world == 1:
        return x
    import torch
    import torch.distributed as dist
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([x], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())


def shard(items, world: int, rank: int):
    """Round-robin share of whole solves for this rank (every item on exactly one rank)."""
    return [it for i, it in enumerate(items) if i % world == rank]
