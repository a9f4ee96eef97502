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


def test_partition_invariants_on_random_costs():
    """Heavy-tailed random costs, 0-59 instances, 1-11 ranks: contiguous ranges in rank
    order covering every instance once, and every boundary within one instance of its
    target, so no rank carries more than total / world + 2 max(cost)."""
    import numpy as np
    from optifax_gb300 import dist
    rng = np.random.default_rng(0)
    for _ in range(2000):
        n, world = int(rng.integers(0, 60)), int(rng.integers(1, 12))
        costs = list(rng.pareto(1.5, size=n) + 0.01)
        parts = dist.partition_by_cost(costs, world)
        assert len(parts) == world
        assert [i for p in parts for i in p] == list(range(n))
        if n:
            bound = sum(costs) / world + 2 * max(costs)
            assert max(sum(costs[i] for i in p) for p in parts) <= bound + 1e-9


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


class _OracleNet:
    """Stand-in for the GPU network with the FP64 oracle's gradients (CPU), for the
    data-parallel step's host logic: backward, set_grads and a plain gradient step."""

    def __init__(self, params, max_batch=4):
        import numpy as np
        self.p = np.array(params, dtype=np.float64)
        self.grad = None
        self.dev = torch.device("cpu")
        self.max_batch = max_batch

    def forward(self, x):
        from oracle import fno_oracle
        return torch.from_numpy(fno_oracle.forward(self.p, x.numpy(), weights_bf16=False)[0].astype("float32"))

    def backward(self, x, target, grads=None, sample_w=None):
        from oracle import fno_oracle
        loss, g, _ = fno_oracle.loss_and_grads(self.p, x.numpy(), target.numpy(), weights_bf16=False,
                                               sample_w=None if sample_w is None else sample_w.numpy())
        self.grad = g
        if grads is not None:
            grads.copy_(torch.from_numpy(g.astype("float32")))
        return torch.tensor([loss], dtype=torch.float32)

    def set_grads(self, grads):
        self.grad = grads.numpy().astype("float64")

    def adam(self, lr, weight_decay=0.0):
        self.p -= lr * self.grad


def _dp_case():
    import numpy as np
    from optifax_gb300 import surrogate
    g = np.random.default_rng(5)
    x = torch.from_numpy(g.standard_normal((4, surrogate.CIN, 64)).astype("float32"))
    t = torch.from_numpy(g.standard_normal((4, surrogate.COUT, 64)).astype("float32"))
    w = torch.from_numpy(g.uniform(0.5, 2.0, 4).astype("float32"))
    return surrogate.init_params(1), x, t, w


def _dp_worker(rank, world, port, out_dir):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    from optifax_gb300 import dist, surrogate
    r, w_, _ = dist.init("gloo")
    params, x, t, w = _dp_case()
    net = _OracleNet(params)
    sl = slice(2 * r, 2 * r + 2)                    # this rank's half of the global batch of 4
    grads = torch.empty(surrogate.N_PARAMS, dtype=torch.float32)
    surrogate.data_parallel_step(net, x[sl], t[sl], 1e-3, sample_w=w[sl], grads=grads)
    got = dist.gather_to_rank0({"rank": r, "p": net.p, "g": grads.numpy().copy()})
    dist.barrier()
    if r == 0:
        import pickle
        with open(os.path.join(out_dir, "dp.pkl"), "wb") as f:
            pickle.dump(got, f)
    torch.distributed.destroy_process_group()


def test_two_rank_data_parallel_surrogate_step():
    """Gradients averaged over 2 ranks (halves of the batch) equal the full-batch
    gradient, and both replicas take the same step."""
    import pickle
    import numpy as np
    from oracle import fno_oracle
    with tempfile.TemporaryDirectory() as d:
        mp.spawn(_dp_worker, args=(2, _free_port(), d), nprocs=2, join=True)
        got = pickle.load(open(os.path.join(d, "dp.pkl"), "rb"))
    params, x, t, w = _dp_case()
    _, g_full, _ = fno_oracle.loss_and_grads(params, x.numpy(), t.numpy(), weights_bf16=False, sample_w=w.numpy())
    for rec in got:
        assert np.allclose(rec["g"], g_full, rtol=1e-4, atol=1e-6 * np.abs(g_full).max())
    assert np.array_equal(got[0]["p"], got[1]["p"])


def _train_case():
    import numpy as np
    from optifax_gb300 import surrogate
    g = np.random.default_rng(7)
    X = torch.from_numpy(g.standard_normal((13, surrogate.CIN, 64)).astype("float32"))
    T = torch.from_numpy((0.5 * g.standard_normal((13, surrogate.COUT, 64))).astype("float32"))
    return surrogate.init_params(3), X, T


def _train_worker(rank, world, port, out_dir):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    from optifax_gb300 import dist, fastforward
    r, _, _ = dist.init("gloo")
    params, X, T = _train_case()
    net = _OracleNet(params)
    fastforward.train(net, X, T, epochs=2, batch=4, lr=1e-3, val_frac=0.1, seed=3)
    got = dist.gather_to_rank0(net.p)
    dist.barrier()
    if r == 0:
        import pickle
        with open(os.path.join(out_dir, "train.pkl"), "wb") as f:
            pickle.dump(got, f)
    torch.distributed.destroy_process_group()


def test_two_rank_training_matches_one_rank():
    """fastforward.train over 2 ranks (each a half of every minibatch, gradients
    averaged) ends with identical replicas equal to the single-rank run."""
    import pickle
    import numpy as np
    from optifax_gb300 import fastforward
    with tempfile.TemporaryDirectory() as d:
        mp.spawn(_train_worker, args=(2, _free_port(), d), nprocs=2, join=True)
        got = pickle.load(open(os.path.join(d, "train.pkl"), "rb"))
    params, X, T = _train_case()
    one = _OracleNet(params)
    fastforward.train(one, X, T, epochs=2, batch=4, lr=1e-3, val_frac=0.1, seed=3)
    assert np.array_equal(got[0], got[1])
    assert np.allclose(got[0], one.p, rtol=1e-5, atol=1e-7)
    assert not np.allclose(one.p, params)
