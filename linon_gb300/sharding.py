"""Sharding across ranks (one process per GPU): views of a batch, or the
rows of one frame.

Rays and views are independent, so a multi-GPU job needs no collective on the
data path: each rank renders the views (or rows) assigned to it.  Views are assigned
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


def shard_rows(height: int, world: int, halo: int = 0):
    """One frame split by rows: per rank (own0, own1, r0, r1), the rank owns
    rows [own0, own1) (contiguous, sizes within one row of each other) and
    renders [r0, r1) = [own0 - halo, own1 + halo) clipped to the image.

    The Lyapunov overlay of a pixel reads the endpoints delta rows above and
    below it and leaves a border of 2 * delta pixels (src/overlay.wgsl:
    114-134).  Run on the rendered band alone with halo = 2 * delta, it
    therefore gives every owned row exactly the value of the whole-frame
    overlay: at an inner edge of the band the skipped border is the halo,
    and where the band is clipped its edge is the image's edge.  No rank
    needs another's rows; the gather is a copy of the owned rows."""
    if world <= 0 or height < 0 or halo < 0:
        raise ValueError("world must be positive, height and halo non-negative")
    out = []
    for k in range(world):
        own0, own1 = height * k // world, height * (k + 1) // world
        out.append((own0, own1, max(0, own0 - halo), min(height, own1 + halo)))
    return out


def overlay_band(engine, field, camera, settings, params, planes, target, exponents, band,
                 srgb: bool = False, fp64: bool = True):
    """Renders a band of shard_rows (halo included) into full-size planes and
    runs the overlay over the band alone; rows [own0, own1) of target and
    exponents then hold the whole-frame values.  The overlay also writes the
    band's halo rows (with the border's pass-through values), so each band
    needs planes and outputs of its own, as each rank has."""
    own0, own1, r0, r1 = band
    engine.render_rows(field, camera, settings, params, planes, r0, r1)
    if r1 > r0:
        engine.overlay(settings, planes.width, r1 - r0, planes.color[r0:r1], planes.mapping[r0:r1],
                       target[r0:r1], None if exponents is None else exponents[r0:r1], srgb=srgb, fp64=fp64)
    return own0, own1
