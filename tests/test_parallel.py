"""Multi-rank sweep logic with world_size 2 over gloo on CPU (no GPU involved).

The ranks' solves are computed by the oracle restatement here (the CPU stands in for each
rank's GPU), so the test covers the partition, the gather back to rank 0 in sweep order and
the reductions; it is unmeasured on GPU hardware (the runs here use one GPU).
"""
import os

import numpy as np
import torch.multiprocessing as mp

from shg_focused_gaussian_beams_gb300 import workloads as W
from shg_focused_gaussian_beams_gb300.parallel import partition_lpt, rank_sweep, solve_cost


def _small_sweep(count=12, seed=5):
    """A sweep with the workload's parameter distributions on small grids (oracle-sized)."""
    out = []
    for i in W.config_sweep(count=count, seed=seed):
        n = {64: 16, 128: 32, 256: 32}[i.nx]
        out.append(W.plain_instance(n, i.nz // 20, i.power, 2.84, i.temp))
    return out


def _oracle_eta(insts):
    import oracle as O
    return list(O.sweep_plain(O.make_cfg(W.CRYSTAL_QPM50, 16, 16, 5), insts, threads=1))


def _worker(rank, world, port, q):
    import sys
    sys.path.insert(0, os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "oracle"))
    import torch.distributed as dist
    from shg_focused_gaussian_beams_gb300.parallel import gather_sweep, world_max, world_sum
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    mine = rank_sweep(16, 5, rank, world, "strong")
    work = sum(i.pt_steps for i in mine)
    insts = _small_sweep()
    idx = partition_lpt(insts, world)[rank]
    eta = _oracle_eta([insts[i] for i in idx])
    fields = [np.full(3, float(i)) for i in idx]
    eta_all, f_all = gather_sweep(idx, eta, len(insts), fields)
    q.put((rank, world_max(10.0 + rank), world_sum(work), work, [(i.nx, i.nz, i.power) for i in mine], eta_all,
           None if f_all is None else [float(f[0]) for f in f_all]))
    dist.barrier()
    dist.destroy_process_group()


def test_gloo_two_ranks_partition_gather_and_reduce():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = 29611
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted((q.get(timeout=180) for _ in range(2)), key=lambda r: r[0])
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert res[0][1] == res[1][1] == 11.0
    total = sum(i.pt_steps for i in rank_sweep(16, 5, 0, 1, "strong"))
    assert res[0][2] == res[1][2] == float(total)
    a, b = set(res[0][4]), set(res[1][4])
    assert not (a & b) and len(a) + len(b) == 16
    # the gathered efficiencies are the one-rank sweep's, in sweep order; rank 1 gets nothing
    insts = _small_sweep()
    assert res[0][5] == _oracle_eta(insts)
    assert res[0][6] == [float(i) for i in range(len(insts))]
    assert res[1][5] is None and res[1][6] is None


def test_lpt_partition_balances_cost():
    insts = W.config_sweep(count=512, seed=2024)
    for world in (2, 4, 8):
        parts = partition_lpt(insts, world)
        assert sorted(i for p in parts for i in p) == list(range(len(insts)))
        loads = [sum(solve_cost(insts[i]) for i in p) for p in parts]
        # LPT is within 4/3 of the optimum; on 512 solves it is within a few per cent
        assert max(loads) / (sum(loads) / world) < 1.02, loads


def test_weak_scaling_ranks_get_distinct_sweeps():
    a = rank_sweep(8, 5, 0, 2)
    b = rank_sweep(8, 5, 1, 2)
    assert len(a) == len(b) == 8 and [i.power for i in a] != [i.power for i in b]


def test_partition_and_gather_edge_cases():
    """More ranks than solves leaves ranks empty (nothing duplicated); an empty sweep gives
    empty parts; on one process the gather returns the sweep order and refuses indices that
    do not cover the sweep."""
    import pytest
    from shg_focused_gaussian_beams_gb300.parallel import gather_sweep
    insts = W.config_sweep(count=3, seed=9)
    parts = partition_lpt(insts, 5)
    assert sorted(i for p in parts for i in p) == [0, 1, 2] and sum(1 for p in parts if not p) == 2
    assert partition_lpt([], 3) == [[], [], []]
    eta, f = gather_sweep([2, 0, 1], [0.3, 0.1, 0.2], 3, fields=["c", "a", "b"])
    assert eta == [0.1, 0.2, 0.3] and f == ["a", "b", "c"]
    assert gather_sweep([1, 0], [0.2, 0.1], 2) == ([0.1, 0.2], None)
    with pytest.raises(ValueError, match="do not cover"):
        gather_sweep([0, 2], [0.1, 0.3], 3)
