"""Sharding of views across ranks (one process per GPU).

Rays and views are independent, so a multi-GPU job needs no collective on the
data path: each rank renders the views assigned to it.  Views are assigned
greedily by ray count (largest first to the least-loaded rank), which keeps
per-rank work within one view of balanced.  The only communication is the
optional gather of per-rank timings / outputs by the caller.
"""
from __future__ import annotations


def shard_views(sizes, world: int):
    """sizes: rays per view.  Returns one list of view indices per rank."""
    if world <= 0:
        raise ValueError("world must be positive")
    order = sorted(range(len(sizes)), key=lambda i: (-sizes[i], i))
    load = [0] * world
    out = [[] for _ in range(world)]
    for i in order:
        r = min(range(world), key=lambda k: (load[k], k))
        out[r].append(i)
        load[r] += sizes[i]
    for lst in out:
        lst.sort()
    return out


def my_views(sizes, rank: int, world: int):
    return shard_views(sizes, world)[rank]
