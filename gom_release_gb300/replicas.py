"""Independent replicas on several GPUs and their aggregate throughput.

One GOM run does not shard across GPUs in this build: N GPUs run N independent replicas (one
process per GPU).  The whole-job figure is the sum of the units all ranks processed divided by the
slowest rank's time; that reduction is the only inter-process communication.
"""
from __future__ import annotations

import os


def world() -> tuple[int, int, int]:
    """(world_size, rank, local_rank) from the torchrun environment (1, 0, 0 without it)."""
    return (int(os.environ.get("WORLD_SIZE", "1")), int(os.environ.get("RANK", "0")),
            int(os.environ.get("LOCAL_RANK", "0")))


def aggregate(units: float, seconds: float, device: str = "cpu") -> tuple[float, float]:
    """Sum of units and maximum of seconds over all ranks of the default process group."""
    import torch
    import torch.distributed as dist
    if not dist.is_available() or not dist.is_initialized():
        return units, seconds
    t = torch.tensor([units, -seconds], dtype=torch.float64, device=device)
    u = t[:1].clone()
    dist.all_reduce(u, op=dist.ReduceOp.SUM)
    m = t[1:].clone()
    dist.all_reduce(m, op=dist.ReduceOp.MIN)
    return float(u.item()), float(-m.item())


def throughput(units: float, seconds: float, device: str = "cpu") -> float:
    total, slowest = aggregate(units, seconds, device)
    return total / slowest
