"""Sharding of independent boxes across ranks, on CPU with the gloo backend (world size 2)."""
import os
import socket

import pytest

from conftest import module


def test_lpt_shard_covers_every_box_once():
    batch = module("batch")
    grf = module("grf")
    specs = grf.uneven_batch()
    costs = [s.n ** 3 for s in specs]
    for world in (1, 2, 3, 8):
        parts = batch.shard(costs, world)
        flat = sorted(i for p in parts for i in p)
        assert flat == list(range(len(specs)))
        loads = [sum(costs[i] for i in p) for p in parts]
        assert max(loads) - min(loads) <= max(costs)


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, q):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    batch = module("batch")
    grf = module("grf")
    specs = grf.uneven_batch()
    parts = batch.shard([s.n ** 3 for s in specs], world)
    mine = parts[rank]
    # each rank "processes" its boxes independently; only scalars are gathered at the end
    results = {i: float(specs[i].n) for i in mine}
    gathered = [None] * world
    dist.all_gather_object(gathered, results)
    if rank == 0:
        merged = {}
        for g in gathered:
            assert not (set(g) & set(merged))
            merged.update(g)
        q.put(sorted(merged))
    dist.destroy_process_group()


def test_two_rank_gloo_shard_gathers_all_boxes():
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    got = q.get(timeout=120)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert got == list(range(len(module("grf").uneven_batch())))
