"""One process per GPU: rank bookkeeping, cost-balanced sharding of independent
crystal passes, max-over-ranks timing and a gather of per-rank results.

Crystal passes of a sweep (and the solver runs that generate surrogate training
pairs) are independent units: each rank takes a contiguous range of instances,
balanced by the cost N log2(N) S (grid points x transform depth x steps), runs it
with no collective on the data path, and rank 0 gathers the results once at the
end.  A single OPO cavity is sequential in round trips, so cavities only run as
independent replicas (one per rank).  Surrogate training is data parallel: each
rank takes its shard of the training pairs and the gradients are averaged over
the ranks every step (all_reduce_mean_).  No reference counterpart: OptiFax runs
on one MATLAB process (its NumOfParRuns pulses share one batched MEX call).
"""
from __future__ import annotations

import math
import os
from typing import List, Optional, Sequence

import torch


def env_rank():
    """(rank, world size, local rank) from the launcher's environment (1 process: 0, 1, 0)."""
    return (int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")),
            int(os.environ.get("LOCAL_RANK", "0")))


def init(backend: str = "nccl"):
    """Initialise the default process group when WORLD_SIZE > 1; returns (rank, world, local)."""
    rank, world, local = env_rank()
    if world > 1 and not torch.distributed.is_initialized():
        torch.distributed.init_process_group(backend)
    return rank, world, local


def pass_cost(n_points: int, n_steps: int) -> float:
    """Relative cost of one crystal pass: N log2(N) S."""
    return float(n_points) * math.log2(max(n_points, 2)) * float(n_steps)


def partition_by_cost(costs: Sequence[float], world: int) -> List[range]:
    """Contiguous ranges of the instances, one per rank, whose cost sums are balanced:
    rank r ends where the running sum first reaches (r + 1) / world of the total
    (whichever side of that point is closer).  Every instance is in exactly one
    range; a rank may get an empty range when there are fewer instances than ranks."""
    n = len(costs)
    if world < 1:
        raise ValueError("world must be >= 1")
    total = float(sum(costs))
    bounds = [0]
    run = 0.0
    i = 0
    for r in range(1, world):
        target = total * r / world
        while i < n and run + costs[i] <= target:
            run += costs[i]
            i += 1
        # include the straddling instance if that lands closer to the target
        if i < n and (run + costs[i] - target) < (target - run) and n - (i + 1) >= world - r:
            run += costs[i]
            i += 1
        bounds.append(max(i, bounds[-1]))
    bounds.append(n)
    return [range(bounds[r], bounds[r + 1]) for r in range(world)]


def max_over_ranks(value: float, device: Optional[torch.device] = None) -> float:
    """Maximum of a per-rank scalar (e.g. a timed region) over all ranks."""
    if not (torch.distributed.is_available() and torch.distributed.is_initialized()):
        return float(value)
    t = torch.tensor([float(value)], dtype=torch.float64, device=device or torch.device("cpu"))
    torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    return float(t.item())


def all_reduce_mean_(t: torch.Tensor) -> torch.Tensor:
    """In place: the mean of `t` over all ranks (a no-op on one rank)."""
    if torch.distributed.is_available() and torch.distributed.is_initialized():
        world = torch.distributed.get_world_size()
        if world > 1:
            torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.SUM)
            t.div_(world)
    return t


def gather_to_rank0(obj) -> Optional[list]:
    """Per-rank Python objects gathered on rank 0 in rank order (None elsewhere)."""
    if not (torch.distributed.is_available() and torch.distributed.is_initialized()):
        return [obj]
    world = torch.distributed.get_world_size()
    out = [None] * world if torch.distributed.get_rank() == 0 else None
    torch.distributed.gather_object(obj, out, dst=0)
    return out


def barrier():
    if torch.distributed.is_available() and torch.distributed.is_initialized():
        torch.distributed.barrier()
