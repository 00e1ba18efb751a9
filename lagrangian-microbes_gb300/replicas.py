"""Replica bookkeeping for multi-GPU runs (one process per GPU, no data-path collective).

The path shards only across independent units (ensembles, or whole replicas of a workload):
a unit never exchanges data with another, so ranks split the units and meet only to agree on
timing (max over ranks) and totals (sum over ranks). This mirrors the reference's process-level
parallelism (joblib tiles, particle_advecter.py:38-66,143-148; SLURM ensembles,
sandbox/slurm_rock_paper_scissors.py) without any collective on the compute path.
"""

from __future__ import annotations


def shard(n_units: int, world: int, rank: int) -> range:
    """Contiguous block of unit indices owned by `rank` (sizes differ by at most one)."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError("need 0 <= rank < world")
    base, extra = divmod(int(n_units), world)
    start = rank * base + min(rank, extra)
    return range(start, start + base + (1 if rank < extra else 0))


def shard_weighted(weights, world: int, rank: int) -> list[int]:
    """Units assigned to `rank` by greedy longest-processing-time balancing of `weights`."""
    order = sorted(range(len(weights)), key=lambda k: (-weights[k], k))
    load = [0.0] * world
    owner = [0] * len(weights)
    for k in order:
        r = min(range(world), key=lambda q: (load[q], q))
        owner[k] = r
        load[r] += weights[k]
    return [k for k in range(len(weights)) if owner[k] == rank]


def _reduce(value: float, op: str) -> float:
    try:
        import torch
        import torch.distributed as dist
    except ImportError:
        return float(value)
    if not (dist.is_available() and dist.is_initialized()):
        return float(value)
    t = torch.tensor([float(value)], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX if op == "max" else dist.ReduceOp.SUM)
    return float(t.item())


def max_over_ranks(value: float) -> float:
    return _reduce(value, "max")


def sum_over_ranks(value: float) -> float:
    return _reduce(value, "sum")
