"""Multi-GPU execution of SU(2) flows: replicas only.

A flow's right-hand side is not split across GPUs: flows are independent (a parameter scan or
a request stream is many flows), so each rank runs whole flows on its own GPU and nothing is
exchanged on the data path.  Ranks meet only to agree on the work split and, for timing, on
the slowest rank's time.  Throughput is the units (cutoff steps or flows) of all ranks divided
by that time (weak scaling).
"""
from __future__ import annotations

from dataclasses import dataclass


def shard(n_items: int, rank: int, world: int) -> list[int]:
    """Items of `rank` when n_items independent flows are dealt round-robin over `world` ranks."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError("bad rank/world")
    return list(range(rank, n_items, world))


@dataclass
class JobTiming:
    units: float      # units processed by all ranks
    seconds: float    # slowest rank's time
    world: int

    @property
    def throughput(self) -> float:
        return self.units / self.seconds if self.seconds > 0 else float("inf")


def aggregate(local_units: float, local_seconds: float, group=None) -> JobTiming:
    """Sums the units and takes the maximum time over the ranks of the default (or given)
    torch.distributed process group; without an initialised group it is the local value."""
    import torch
    import torch.distributed as dist

    if not (dist.is_available() and dist.is_initialized()):
        return JobTiming(float(local_units), float(local_seconds), 1)
    backend = dist.get_backend(group)
    device = torch.device("cuda", torch.cuda.current_device()) if backend == "nccl" else torch.device("cpu")
    units = torch.tensor([float(local_units)], dtype=torch.float64, device=device)
    secs = torch.tensor([float(local_seconds)], dtype=torch.float64, device=device)
    dist.all_reduce(units, op=dist.ReduceOp.SUM, group=group)
    dist.all_reduce(secs, op=dist.ReduceOp.MAX, group=group)
    return JobTiming(float(units.item()), float(secs.item()), dist.get_world_size(group))


def _rank_world(group=None) -> tuple[int, int]:
    import torch.distributed as dist

    if dist.is_available() and dist.is_initialized():
        return dist.get_rank(group), dist.get_world_size(group)
    return 0, 1


def run_sharded(items: list, solve, group=None):
    """Runs independent flows on all ranks: the items are dealt round-robin (``shard``), each
    rank calls ``solve(local_items) -> (results, seconds)`` on its own GPU, and the results are
    gathered on every rank in the items' order.  Nothing crosses ranks on the data path: the
    only exchanges are the two scalars of ``aggregate`` and the gathered results after the
    timed work.  Returns (JobTiming over all ranks, results[len(items)], local indices)."""
    import torch.distributed as dist

    rank, world = _rank_world(group)
    mine = shard(len(items), rank, world)
    results, seconds = solve([items[i] for i in mine])
    if len(results) != len(mine):
        raise ValueError("solve returned a different number of results than items")
    job = aggregate(len(mine), seconds, group)
    out = [None] * len(items)
    if world == 1:
        parts = [(mine, results)]
    else:
        parts = [None] * world
        dist.all_gather_object(parts, (mine, results), group=group)
    for idx, res in parts:
        for i, r in zip(idx, res):
            out[i] = r
    return job, out, mine
