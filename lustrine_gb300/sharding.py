"""Scene sharding across processes (one GPU each) for batches of independent
scenes.

Scenes never interact, so a batch shards by scene with no collective on the
data path: every rank builds one batched context from its own scenes and
steps it; only scalar statistics (the FP64 reductions) are gathered on the
host at the end.  The partition is deterministic (every rank computes the
same one from the scene sizes alone) and balances particles: longest
processing time first, each scene to the rank with the fewest particles so
far (ties to the lower rank), which keeps every rank within the largest
scene of the mean.
"""
from __future__ import annotations

import heapq


def shard_scenes(counts, world: int) -> list[list[int]]:
    """Scene indices of every rank, each list ascending."""
    if world < 1:
        raise ValueError("world must be >= 1")
    order = sorted(range(len(counts)), key=lambda i: (-int(counts[i]), i))
    heap = [(0, r) for r in range(world)]
    heapq.heapify(heap)
    out = [[] for _ in range(world)]
    for i in order:
        load, r = heapq.heappop(heap)
        out[r].append(i)
        heapq.heappush(heap, (load + int(counts[i]), r))
    return [sorted(s) for s in out]


def my_scenes(counts, world: int, rank: int) -> list[int]:
    return shard_scenes(counts, world)[rank]


def combine_reductions(parts) -> dict:
    """Combine per-rank FP64 reductions (PbfSim.reduce() dicts) into the
    whole batch's: masses, momenta and kinetic energies add, the centre of
    mass is the mass-weighted mean, the density error the maximum."""
    parts = [p for p in parts if p is not None and p["mass"] > 0]
    if not parts:
        return {"mass": 0.0, "momentum": [0.0, 0.0, 0.0], "kinetic": 0.0, "com": [0.0, 0.0, 0.0],
                "max_density_error": 0.0}
    m = sum(p["mass"] for p in parts)
    return {
        "mass": m,
        "momentum": [sum(p["momentum"][a] for p in parts) for a in range(3)],
        "kinetic": sum(p["kinetic"] for p in parts),
        "com": [sum(p["com"][a] * p["mass"] for p in parts) / m for a in range(3)],
        "max_density_error": max(p["max_density_error"] for p in parts),
    }


def gather_reductions(local: dict | None, world: int) -> dict:
    """Host-side gather of every rank's reductions (torch.distributed object
    gather; the only cross-rank traffic of a sharded batch)."""
    if world == 1:
        return combine_reductions([local])
    import torch.distributed as dist
    parts = [None] * world
    dist.all_gather_object(parts, local)
    return combine_reductions(parts)
