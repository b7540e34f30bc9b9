"""Sharding of ensembles across ranks (one process per GPU).

The runs of an ensemble are independent, so ranks share no data while they
step: each rank builds its own ``Ensemble`` from its shard of the global run
list, and the only exchanges are host-side scalars after the timed region --
the maximum of the ranks' times and a gather of per-run error scalars to
rank 0.  A single grid does not shard (its 2D transform would need a global
transpose), so N ranks of the single-grid solver are replicas.

The functions take the process group module (``torch.distributed``) or None
for one process, and work over ``gloo`` as over ``nccl``.
"""
from __future__ import annotations

import math


def run_cost(n: int) -> float:
    """Relative cost of one step of an n x n run: its transforms, n^2 log2 n."""
    return float(n) * n * math.log2(max(2, n))


def partition_runs(sizes, world_size: int) -> list[list[int]]:
    """Split runs of the given grid sizes over world_size ranks by cost.

    Longest-processing-time order: runs by decreasing cost (ties by index) go
    to the least-loaded rank (ties to the lower rank).  Every index lands on
    exactly one rank; each shard lists its indices in increasing order, so a
    one-rank partition keeps the global order.  With equal counts of each size
    divisible by world_size, every rank gets the same mix of sizes."""
    if world_size < 1:
        raise ValueError("world_size must be >= 1")
    sizes = [int(n) for n in sizes]
    load = [0.0] * world_size
    shards: list[list[int]] = [[] for _ in range(world_size)]
    for i in sorted(range(len(sizes)), key=lambda i: (-run_cost(sizes[i]), i)):
        r = min(range(world_size), key=lambda r: (load[r], r))
        shards[r].append(i)
        load[r] += run_cost(sizes[i])
    return [sorted(s) for s in shards]


def shard_of(runs, rank: int, world_size: int):
    """(global indices, runs) of this rank's shard of a list of (n, k0, seed)."""
    idx = partition_runs([r[0] for r in runs], world_size)[rank]
    return idx, [runs[i] for i in idx]


def _device_for(dist):
    """Tensors for collectives live on the GPU under nccl, on the host otherwise."""
    import torch

    if dist is not None and dist.get_backend() == "nccl":
        return torch.device("cuda", torch.cuda.current_device())
    return torch.device("cpu")


def max_over_ranks(x: float, dist=None) -> float:
    """The largest of the ranks' values of x (every rank gets it)."""
    if dist is None:
        return float(x)
    import torch

    t = torch.tensor([float(x)], dtype=torch.float64, device=_device_for(dist))
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def sum_over_ranks(x: float, dist=None) -> float:
    """The sum of the ranks' values of x (every rank gets it)."""
    if dist is None:
        return float(x)
    import torch

    t = torch.tensor([float(x)], dtype=torch.float64, device=_device_for(dist))
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())


def gather_by_index(indices, values, total: int, dist=None):
    """Per-run scalars of all shards in global order, on rank 0 (None elsewhere).

    indices and values are this rank's global run indices and their scalars.
    Raises ValueError on rank 0 when the shards do not cover 0..total-1 exactly
    once."""
    indices, values = [int(i) for i in indices], [float(v) for v in values]
    if len(indices) != len(values):
        raise ValueError("indices and values differ in length")
    if dist is None:
        parts = [(indices, values)]
        rank = 0
    else:
        rank = dist.get_rank()
        parts = [None] * dist.get_world_size()
        dist.all_gather_object(parts, (indices, values))
    if rank != 0:
        return None
    out = [None] * total
    for idx, vals in parts:
        for i, v in zip(idx, vals):
            if not 0 <= i < total or out[i] is not None:
                raise ValueError(f"run {i} is outside 0..{total - 1} or reported twice")
            out[i] = v
    missing = [i for i, v in enumerate(out) if v is None]
    if missing:
        raise ValueError(f"runs {missing[:8]} were reported by no rank")
    return out
