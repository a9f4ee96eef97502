"""Sharding, timing and gather of independent crystal passes over 2 ranks (gloo, CPU)."""
import os
import socket
import tempfile

import pytest
import torch
import torch.multiprocessing as mp


def test_partition_balances_and_covers():
    from optifax_gb300 import dist, sweep
    insts = sweep.uneven_sweep_instances(n=64, seed=2)
    from optifax_gb300 import physics as ph
    costs = [dist.pass_cost(i.n_points, ph.Crystal(i.length, i.period).n_steps) for i in insts]
    for world in (1, 2, 3, 8):
        parts = dist.partition_by_cost(costs, world)
        assert len(parts) == world
        idx = [i for p in parts for i in p]
        assert idx == list(range(len(insts)))                 # contiguous, each exactly once
        loads = [sum(costs[i] for i in p) for p in parts]
        assert max(loads) - min(loads) <= max(costs) + 1e-9   # within one instance of balance
    assert [len(p) for p in dist.partition_by_cost([1.0], 2)] in ([1, 0], [0, 1])


def _worker(rank, world, port, out_dir):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    from optifax_gb300 import dist
    r, w, _ = dist.init("gloo")
    costs = [float(c) for c in range(1, 21)]
    part = dist.partition_by_cost(costs, w)[r]
    local = {"rank": r, "items": list(part), "work": sum(costs[i] for i in part)}
    t = dist.max_over_ranks(10.0 + r)
    got = dist.gather_to_rank0(local)
    dist.barrier()
    if r == 0:
        with open(os.path.join(out_dir, "result.txt"), "w") as f:
            f.write(repr({"t": t, "got": got}))
    torch.distributed.destroy_process_group()


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_two_rank_shard_gather_and_max_time():
    with tempfile.TemporaryDirectory() as d:
        mp.spawn(_worker, args=(2, _free_port(), d), nprocs=2, join=True)
        res = eval(open(os.path.join(d, "result.txt")).read())
    assert res["t"] == 11.0                                   # the slower rank's time
    got = res["got"]
    assert [g["rank"] for g in got] == [0, 1]
    assert got[0]["items"] + got[1]["items"] == list(range(20))
    assert abs(got[0]["work"] - got[1]["work"]) <= 20
