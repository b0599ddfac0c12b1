"""Sharding independent work across ranks (one process per GPU).

The operator itself does not shard: one system's mesh lives on one GPU (a
distributed FFT would need all-to-all transposes, which this project does not
do).  What shards is independent work:

* a batch of independent systems of uneven size (N, K, p) — partitioned by
  estimated cost with the longest-processing-time rule, no data exchange;
* the right-hand sides of one system — contiguous blocks per rank, every
  rank holding the same positions.

Results are gathered on the host (``torch.distributed`` object collectives on
any backend, ``gloo`` in the CPU tests); there is no device collective on the
data path.
"""
from __future__ import annotations

import math
from typing import Callable, Sequence


def system_cost(n: int, K: int, p: int, nrhs: int, neighbours: float = 40.0) -> float:
    """Relative cost of one apply: spread/interpolate (n p^3 per component), the
    3D FFTs (K^3 log K per component) and the real-space pairs."""
    C = 3 * nrhs
    return 2.0 * n * p ** 3 * C + 5.0 * K ** 3 * math.log2(max(K, 2) ** 3) * C / 3.0 \
        + 20.0 * n * neighbours * nrhs


def partition(costs: Sequence[float], world: int) -> list[list[int]]:
    """Longest-processing-time assignment of items to `world` ranks.

    Deterministic: ties broken by item index, then by rank.  Every item is
    assigned exactly once; the heaviest rank exceeds the mean load by at most
    the largest single item."""
    if world < 1:
        raise ValueError("world must be >= 1")
    order = sorted(range(len(costs)), key=lambda i: (-costs[i], i))
    load = [0.0] * world
    parts: list[list[int]] = [[] for _ in range(world)]
    for i in order:
        r = min(range(world), key=lambda k: (load[k], k))
        parts[r].append(i)
        load[r] += costs[i]
    for p in parts:
        p.sort()
    return parts


def split_rhs(nrhs: int, world: int) -> list[tuple[int, int]]:
    """Contiguous [begin, end) blocks of right-hand sides, sizes differing by <= 1."""
    base, extra = divmod(nrhs, world)
    out, b = [], 0
    for r in range(world):
        e = b + base + (1 if r < extra else 0)
        out.append((b, e))
        b = e
    return out


def run_sharded(items: Sequence, costs: Sequence[float], apply_fn: Callable, dist=None):
    """Run apply_fn(item) for this rank's share of `items` and gather every
    result on rank 0 in item order (other ranks return None).  Without a
    process group (dist None or not initialised) everything runs locally."""
    if dist is None or not dist.is_available() or not dist.is_initialized():
        return [apply_fn(it) for it in items]
    world, rank = dist.get_world_size(), dist.get_rank()
    mine = partition(costs, world)[rank]
    local = {i: apply_fn(items[i]) for i in mine}
    gathered = [None] * world if rank == 0 else None
    dist.gather_object(local, gathered, dst=0)
    if rank != 0:
        return None
    merged: dict = {}
    for part in gathered:
        merged.update(part)
    return [merged[i] for i in range(len(items))]
