"""Multi-process sharding over gloo (CPU, world size 2): views of a batch,
and the rows of one frame (the halo rule of the overlay, checked with the
oracle)."""
import os
import socket

import numpy as np
import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp

from linon_gb300 import sharding, workloads as wl


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, sizes, q):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    mine = sharding.my_views(sizes, rank, world)
    work = torch.tensor([sum(sizes[i] for i in mine)], dtype=torch.int64)
    lists = [None] * world
    dist.all_gather_object(lists, mine)
    works = [torch.zeros(1, dtype=torch.int64) for _ in range(world)]
    dist.all_gather(works, work)
    if rank == 0:
        q.put((lists, [int(w.item()) for w in works]))
    dist.barrier()
    dist.destroy_process_group()


def test_views_partitioned_across_two_ranks():
    sizes = [w * h for (w, h, _, _, _) in wl.batch_views(64, seed=0)]
    port = _free_port()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, sizes, q)) for r in range(2)]
    for p in procs:
        p.start()
    lists, works = q.get(timeout=120)
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    flat = sorted(i for lst in lists for i in lst)
    assert flat == list(range(len(sizes)))          # complete and disjoint
    assert max(works) - min(works) <= max(sizes)    # balanced within one view


def test_shard_views_edge_cases():
    assert sharding.shard_views([], 3) == [[], [], []]
    assert sharding.shard_views([5], 2) == [[0], []]
    with pytest.raises(ValueError):
        sharding.shard_views([1], 0)


# ---- one frame split by rows (halo of 2 * delta for the overlay) ----

def _frame_for_overlay(W=40, H=37):
    """The oracle's rendered planes of a small Lyapunov-style frame."""
    from oracle import pyoracle
    w = wl.lyapunov_1024(W, H)
    w.params = wl.fixed_steps(0.01, 60)
    r = pyoracle.render(w.xyz, w.faces, w.face_rgb, w.camera, w.settings, w.params, w.fields[0], W, H,
                        want=("color", "mapping"))
    return pyoracle, r["color"].reshape(H, W, 4), r["mapping"].reshape(H, W, 4), W, H


def test_shard_rows_partition():
    for H, world, halo in ((37, 2, 4), (37, 5, 2), (3, 4, 1), (0, 2, 3), (100, 1, 6)):
        bands = sharding.shard_rows(H, world, halo)
        assert len(bands) == world
        owned = [r for (o0, o1, _, _) in bands for r in range(o0, o1)]
        assert owned == list(range(H))                                  # complete, disjoint, in order
        sizes = [o1 - o0 for (o0, o1, _, _) in bands]
        assert max(sizes) - min(sizes) <= 1
        for (o0, o1, r0, r1) in bands:
            assert r0 == max(0, o0 - halo) and r1 == min(H, o1 + halo)
    with pytest.raises(ValueError):
        sharding.shard_rows(10, 0)


@pytest.mark.parametrize("world,delta,precision", [(2, 1, 32), (3, 2, 64), (5, 1, 64)])
def test_row_shards_overlay_equals_whole_frame(world, delta, precision):
    """The overlay of each band alone (halo 2 * delta) gives the owned rows
    of the whole-frame overlay bit for bit (oracle, CPU)."""
    pyoracle, color, mapping, W, H = _frame_for_overlay()
    st = wl.settings(overlay_mode=1, delta=delta, scaling=20.0)
    whole, e_whole = pyoracle.overlay(color, mapping, W, H, st, precision=precision)
    for (o0, o1, r0, r1) in sharding.shard_rows(H, world, 2 * delta):
        out, e = pyoracle.overlay(color[r0:r1], mapping[r0:r1], W, r1 - r0, st, precision=precision)
        np.testing.assert_array_equal(out[o0 - r0:o1 - r0], whole[o0:o1])
        np.testing.assert_array_equal(e[o0 - r0:o1 - r0], e_whole[o0:o1])
    # a halo of delta alone is not enough: inner band edges lose 2 * delta rows
    bands = sharding.shard_rows(H, 2, delta)
    o0, o1, r0, r1 = bands[1]
    _, e = pyoracle.overlay(color[r0:r1], mapping[r0:r1], W, r1 - r0, st, precision=precision)
    assert not np.array_equal(e[o0 - r0:o1 - r0], e_whole[o0:o1])


def _row_worker(rank, world, port, q):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    pyoracle, color, mapping, W, H = _frame_for_overlay()
    st = wl.settings(overlay_mode=1, delta=2, scaling=20.0)
    o0, o1, r0, r1 = sharding.shard_rows(H, world, 4)[rank]
    _, e = pyoracle.overlay(color[r0:r1], mapping[r0:r1], W, r1 - r0, st, precision=64)
    mine = torch.from_numpy(np.ascontiguousarray(e[o0 - r0:o1 - r0]))
    parts = [None] * world
    dist.all_gather_object(parts, mine)                  # the gather: owned rows only
    if rank == 0:
        _, e_whole = pyoracle.overlay(color, mapping, W, H, st, precision=64)
        q.put(bool(np.array_equal(torch.cat(parts).numpy(), e_whole)))
    dist.barrier()
    dist.destroy_process_group()


def test_row_shards_over_two_ranks():
    port = _free_port()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_row_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    ok = q.get(timeout=180)
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    assert ok
