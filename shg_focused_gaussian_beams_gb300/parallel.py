"""Rank-level work split for sweeps on several GPUs (one process per GPU).

Solves are independent, so ranks share no data: in weak scaling every rank runs its own
seeded sweep (seed + rank); in strong scaling the solves of one sweep are dealt to ranks
round-robin by descending cost. The only cross-rank traffic is the reduction of timings
and counters (max / sum), over whatever torch.distributed group is initialised (NCCL on
GPUs, gloo on CPU).
"""
from __future__ import annotations

from . import workloads as W


def rank_sweep(count: int, seed: int, rank: int, world: int, scaling: str = "weak"):
    """The solves rank `rank` of `world` runs."""
    if scaling == "weak":
        return W.config_sweep(count=count, seed=seed + rank)
    insts = W.config_sweep(count=count, seed=seed)
    order = sorted(range(len(insts)), key=lambda i: -insts[i].pt_steps)
    return [insts[i] for k, i in enumerate(order) if k % world == rank]


def _reduce(value: float, op: str) -> float:
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(value)
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([float(value)], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX if op == "max" else dist.ReduceOp.SUM)
    return float(t.item())


def world_max(value: float) -> float:
    return _reduce(value, "max")


def world_sum(value: float) -> float:
    return _reduce(value, "sum")
