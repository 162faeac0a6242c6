"""One process per GPU: how the work of a multi-GPU run is split and how the
per-rank results are combined.

A single chamber does not shard (a halo exchange every FTCS substep and a
cross-device transmittance scan would be needed), so single-chamber runs are
replicas: every rank advances its own chamber and the job's rate is the sum of
the ranks' work over the slowest rank's time. A batch of independent chambers
shards with no collective on the data path: chambers go heaviest first to the
least-loaded rank. The only collectives are these scalar reductions at report
time (NCCL on GPUs, gloo on CPU).
"""


def lpt_shards(costs, world_size):
    """Chamber indices per rank: heaviest first onto the least-loaded rank
    (ties by lower index), so every rank gets a deterministic, disjoint share."""
    order = sorted(range(len(costs)), key=lambda i: (-costs[i], i))
    load = [0.0] * world_size
    shards = [[] for _ in range(world_size)]
    for i in order:
        r = min(range(world_size), key=lambda k: (load[k], k))
        shards[r].append(i)
        load[r] += costs[i]
    return [sorted(s) for s in shards]


def _tensor(dist, v):
    import torch
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    return torch.tensor([float(v)], dtype=torch.float64, device=dev)


def reduce_max(dist, v):
    """Largest v over ranks (dist None: single process)."""
    if dist is None:
        return float(v)
    t = _tensor(dist, v)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def reduce_sum(dist, v):
    """Sum of v over ranks."""
    if dist is None:
        return float(v)
    t = _tensor(dist, v)
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())


def job_rate(dist, units, seconds):
    """Whole-job rate: all ranks' units over the slowest rank's time."""
    return reduce_sum(dist, units) / reduce_max(dist, seconds)
