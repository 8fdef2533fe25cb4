"""Sharding of independent boxes across ranks, on CPU with the gloo backend (world size 2).

Boxes weigh N^3 * N_R (voxels times filter radii).  The two-rank test runs real host-path work:
every rank builds the ionisation setups of its share of small boxes, runs the FP64 oracle on
them and only the per-box scalars (neutral fraction, mean x_HI) travel, gathered on rank 0 and
checked against a serial run of the whole batch.
"""
import os
import socket

import numpy as np
import pytest

from conftest import module


def test_box_cost_is_voxels_times_radii():
    batch = module("batch")
    sch = module("schedule")
    cos = module("cosmology")
    grf = module("grf")
    specs = grf.uneven_batch()
    parts = batch.shard_specs(specs, 2)
    n_r = [sch.ionize_setup(s.n, s.box_len, s.z, zeta=s.zeta, t_vir_min=s.t_vir_min, R_max=s.R_max,
                            cosmo=cos.BASELINE_COSMO).n_radii for s in specs]
    costs = [s.n ** 3 * r for s, r in zip(specs, n_r)]
    assert [batch.box_cost(s.n, r) for s, r in zip(specs, n_r)] == costs
    # same n, different R_mfp: different radius counts, so different weights
    same_n = {}
    for s, r in zip(specs, n_r):
        same_n.setdefault(s.n, set()).add(r)
    assert any(len(v) > 1 for v in same_n.values())
    assert parts == batch.shard(costs, 2)


def test_lpt_shard_covers_every_box_once():
    batch = module("batch")
    grf = module("grf")
    specs = grf.uneven_batch()
    sch = module("schedule")
    cos = module("cosmology")
    costs = [batch.box_cost(s.n, sch.ionize_setup(s.n, s.box_len, s.z, zeta=s.zeta, t_vir_min=s.t_vir_min,
                                                  R_max=s.R_max, cosmo=cos.BASELINE_COSMO).n_radii)
             for s in specs]
    for world in (1, 2, 3, 8):
        parts = batch.shard(costs, world)
        flat = sorted(i for p in parts for i in p)
        assert flat == list(range(len(specs)))
        loads = [sum(costs[i] for i in p) for p in parts]
        assert max(loads) - min(loads) <= max(costs)


def test_weak_scaling_sweep_gives_every_rank_a_full_sweep():
    # bench.py --gpus N: 4 seeds x 13 redshifts per GPU, split by cost; every box costs the same
    batch = module("batch")
    grf = module("grf")
    for world in (1, 2, 4, 8):
        specs = grf.sweep_256(seeds=range(4 * world))
        parts = batch.shard([batch.box_cost(256, 32)] * len(specs), world)
        assert [len(p) for p in parts] == [52] * world


def _small_specs():
    grf = module("grf")
    rng = np.random.Generator(np.random.PCG64(7))
    out = []
    for i in range(10):
        n = int(rng.choice([16, 24]))
        out.append(grf.BoxSpec(n, 1.5 * n, 500 + i, float(rng.uniform(6.0, 10.0)), float(rng.uniform(10.0, 80.0)),
                               float(rng.uniform(5.0, 20.0)), float(10 ** rng.uniform(4.0, 5.0))))
    return out


def _run_box(spec):
    """Host path of one box: ionisation setup, density, FP64 oracle; returns (nf, x_HI mean)."""
    from oracle import es_oracle as O
    grf = module("grf")
    sch = module("schedule")
    cos = module("cosmology")
    st = sch.ionize_setup(spec.n, spec.box_len, spec.z, zeta=spec.zeta, t_vir_min=spec.t_vir_min,
                          R_max=spec.R_max, cosmo=cos.BASELINE_COSMO)
    d = grf.density_box(spec.n, spec.box_len, spec.seed, spec.z)
    ion = O.conv_bubbles(d, st)["ionized"]
    return st.n_radii, float(1.0 - ion.mean())


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
    specs = _small_specs()
    mine = batch.shard_specs(specs, world)[rank]
    # every rank processes its own boxes; only scalars are gathered, no data-path collective
    results = {i: _run_box(specs[i]) for i in mine}
    gathered = [None] * world
    dist.all_gather_object(gathered, results)
    if rank == 0:
        merged = {}
        for g in gathered:
            assert not (set(g) & set(merged))
            merged.update(g)
        q.put(merged)
    dist.destroy_process_group()


def test_two_rank_gloo_shard_runs_boxes_and_gathers_scalars():
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    got = q.get(timeout=300)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    specs = _small_specs()
    assert sorted(got) == list(range(len(specs)))
    serial = {i: _run_box(s) for i, s in enumerate(specs)}
    assert got == serial                       # same arithmetic on every rank: identical scalars
    assert len({v[0] for v in serial.values()}) > 1
