"""One process per GPU: partitioning of independent problem instances across
ranks and the host-side reductions of the timing and metrics.

The path has no exchange step: batched instances (different parameters and
meshes) are independent, so rank r advances its share of the instances on
its own GPU and only scalars cross ranks (the slowest rank's time, summed
work counts).  A single large mesh is replicated on every rank, not split.
"""
from __future__ import annotations


def shard_by_cost(costs, world):
    """Deterministic partition of instance indices into `world` shards with
    balanced total cost (greedy: largest first onto the least-loaded shard,
    ties to the lower rank); each shard keeps its indices in ascending order."""
    order = sorted(range(len(costs)), key=lambda i: (-costs[i], i))
    load = [0.0] * world
    shards = [[] for _ in range(world)]
    for i in order:
        r = min(range(world), key=lambda k: (load[k], k))
        shards[r].append(i)
        load[r] += costs[i]
    return [sorted(s) for s in shards]


def gather_instances(mine, arrays, n_instances):
    """Reassemble per-instance results computed on the ranks: rank r passes
    its shard `mine` (instance indices) and the matching host arrays; every
    rank receives the list of all n_instances arrays in global instance
    order.  Each instance must be owned by exactly one rank."""
    import torch.distributed as dist
    local = list(zip((int(i) for i in mine), arrays))
    if dist.is_available() and dist.is_initialized() and dist.get_world_size() > 1:
        parts = [None] * dist.get_world_size()
        dist.all_gather_object(parts, local)
    else:
        parts = [local]
    out = [None] * n_instances
    for part in parts:
        for i, a in part:
            if out[i] is not None:
                raise ValueError(f"instance {i} owned by more than one rank")
            out[i] = a
    missing = [i for i, a in enumerate(out) if a is None]
    if missing:
        raise ValueError(f"instances without an owner: {missing[:8]}")
    return out


def max_over_ranks(value, device=None):
    """The largest value over all ranks (a step's time is the slowest rank's)."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(value)
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def sum_over_ranks(value, device=None):
    """The sum over all ranks (work done by the whole job)."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(value)
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())
