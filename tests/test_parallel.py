"""Multi-rank sweep logic with world_size 2 over gloo on CPU (no GPU involved)."""
import os

import pytest
import torch.multiprocessing as mp

from shg_focused_gaussian_beams_gb300.parallel import rank_sweep


def _worker(rank, world, port, q):
    import torch.distributed as dist
    from shg_focused_gaussian_beams_gb300.parallel import world_max, world_sum
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    mine = rank_sweep(16, 5, rank, world, "strong")
    work = sum(i.pt_steps for i in mine)
    q.put((rank, world_max(10.0 + rank), world_sum(work), work, [(i.nx, i.nz, i.power) for i in mine]))
    dist.barrier()
    dist.destroy_process_group()


def test_gloo_two_ranks_reduce_and_shard():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = 29611
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in range(2))
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert res[0][1] == res[1][1] == 11.0
    total = sum(i.pt_steps for i in rank_sweep(16, 5, 0, 1, "strong"))
    assert res[0][2] == res[1][2] == float(total)
    a, b = set(res[0][4]), set(res[1][4])
    assert not (a & b) and len(a) + len(b) == 16
    assert abs(res[0][3] - res[1][3]) / total < 0.25  # balanced by cost


def test_weak_scaling_ranks_get_distinct_sweeps():
    a = rank_sweep(8, 5, 0, 2)
    b = rank_sweep(8, 5, 1, 2)
    assert len(a) == len(b) == 8 and [i.power for i in a] != [i.power for i in b]
