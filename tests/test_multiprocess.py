"""Multi-process view sharding over gloo (CPU, world size 2)."""
import os
import socket

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
