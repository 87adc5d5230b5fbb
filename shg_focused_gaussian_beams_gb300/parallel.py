"""Rank-level work split for sweeps on several GPUs (one process per GPU).

Solves are independent (the reference runs one process per sweep point, SHG.sh:81), so
ranks share no field data while they march:

* weak scaling: every rank runs its own seeded sweep (seed + rank);
* strong scaling: the solves of one sweep are partitioned over the ranks by estimated cost
  (longest-processing-time-first: each solve, costliest first, goes to the least-loaded
  rank), and rank 0 gathers the efficiencies (and, on request, the output fields) back in
  sweep order.

The cost of a solve is the method's flop count, N^2 Nz (20 log2(N^2) + 456): four 2D FFTs
at 5 N^2 log2(N^2) each plus the two RK4 calls and propagator products per grid point and
z-step. Cross-rank traffic is the gather and the reduction of timings and counters (max /
sum), over whatever torch.distributed group is initialised (NCCL on GPUs, gloo on CPU).
"""
from __future__ import annotations

import heapq
import math

from . import workloads as W


def solve_cost(inst) -> float:
    """Estimated work of one solve (flops of the method)."""
    nn = inst.nx * inst.ny
    return float(nn) * inst.nz * (20.0 * math.log2(nn) + 456.0)


def partition_lpt(insts, world: int) -> list[list[int]]:
    """Indices of `insts` per rank: costliest solve first to the least-loaded rank (ties go
    to the lower rank); every rank's list is in ascending sweep order."""
    heap = [(0.0, r) for r in range(world)]
    parts: list[list[int]] = [[] for _ in range(world)]
    for i in sorted(range(len(insts)), key=lambda i: (-solve_cost(insts[i]), i)):
        load, r = heapq.heappop(heap)
        parts[r].append(i)
        heapq.heappush(heap, (load + solve_cost(insts[i]), r))
    return [sorted(p) for p in parts]


def rank_indices(count: int, seed: int, rank: int, world: int) -> list[int]:
    """Strong scaling: the sweep indices rank `rank` of `world` runs."""
    return partition_lpt(W.config_sweep(count=count, seed=seed), world)[rank]


def rank_sweep(count: int, seed: int, rank: int, world: int, scaling: str = "weak"):
    """The solves rank `rank` of `world` runs."""
    if scaling == "weak":
        return W.config_sweep(count=count, seed=seed + rank)
    insts = W.config_sweep(count=count, seed=seed)
    return [insts[i] for i in partition_lpt(insts, world)[rank]]


def _dist():
    import torch.distributed as dist
    return dist if dist.is_available() and dist.is_initialized() and dist.get_world_size() > 1 else None


def gather_sweep(indices, eta, count: int, fields=None):
    """Strong scaling: every rank passes the sweep indices it ran, their efficiencies and
    optionally their output fields (a list of arrays in the same order); rank 0 receives the
    efficiencies of the whole sweep in sweep order (a list of `count` floats) and the fields
    (a list of `count` arrays, or None), the other ranks receive (None, None). Works on one
    process too (no group: the inputs are returned in sweep order)."""
    local = (list(indices), [float(e) for e in eta], None if fields is None else list(fields))
    dist = _dist()
    if dist is None:
        parts = [local]
    else:
        parts = [None] * dist.get_world_size() if dist.get_rank() == 0 else None
        dist.gather_object(local, parts, dst=0)
        if dist.get_rank() != 0:
            return None, None
    eta_all = [None] * count
    f_all = [None] * count if fields is not None else None
    for idx, e, f in parts:
        for k, i in enumerate(idx):
            eta_all[i] = e[k]
            if f_all is not None and f is not None:
                f_all[i] = f[k]
    if any(v is None for v in eta_all):
        raise ValueError("gather_sweep: the ranks' indices do not cover the sweep")
    return eta_all, f_all


def _reduce(value: float, op: str) -> float:
    import torch
    dist = _dist()
    if dist is None:
        return float(value)
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([float(value)], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX if op == "max" else dist.ReduceOp.SUM)
    return float(t.item())


def world_max(value: float) -> float:
    return _reduce(value, "max")


def world_sum(value: float) -> float:
    return _reduce(value, "sum")
