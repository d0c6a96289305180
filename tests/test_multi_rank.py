"""CPU, two gloo ranks: the multi-GPU host logic of the bench.  Cloths are independent,
so ranks shard by cloth with no collective on the data path; the only collectives are
the timing max and the barrier around the timed region.  A second test has each rank
simulate its shard (with the oracle standing in for the GPU solver, so that it runs on
CPU) and checks that the gathered cloths equal the whole batch simulated in one
process."""
import os
import socket

import numpy as np
import pytest
import torch.distributed as dist
import torch.multiprocessing as mp

from velvet_gb300 import workloads as W


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        wl = W.batched(64, frames=1, seed=3)
        mine = W.shard(wl, rank, world)
        ids = [id_ for id_, c in enumerate(wl.cloths) if any(c is m for m in mine.cloths)]
        gathered = [None] * world
        dist.all_gather_object(gathered, ids)
        # the bench's aggregation: total work over the slowest rank's time
        import torch

        elapsed = torch.tensor([1.0 + rank], dtype=torch.float64)
        dist.all_reduce(elapsed, op=dist.ReduceOp.MAX)
        work = torch.tensor([float(sum(c.num_particles for c in mine.cloths))], dtype=torch.float64)
        dist.all_reduce(work, op=dist.ReduceOp.SUM)
        if rank == 0:
            q.put((gathered, float(elapsed.item()), float(work.item()), wl.num_particles))
    finally:
        dist.destroy_process_group()


def _simulate_worker(rank, world, port, q):
    import sys
    from pathlib import Path

    sys.path.insert(0, str(Path(__file__).resolve().parent))
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        from oracle import Oracle

        wl = W.batched(12, frames=2, seed=5, lo=6, hi=14)
        mine = W.shard(wl, rank, world)
        ids = [id_ for id_, c in enumerate(wl.cloths) if any(c is m for m in mine.cloths)]
        out = {}
        for id_, spec in zip(ids, mine.cloths):
            o = Oracle()
            W.build_plain(spec, o)
            for _ in range(wl.frames):
                o.simulate(wl.frame_dt, wl.substeps, wl.iterations, wl.relaxation, wl.friction,
                           wl.collision_margin, spec.particle_diameter())
            out[id_] = o.positions().tobytes()
        gathered = [None] * world
        dist.all_gather_object(gathered, out)
        if rank == 0:
            q.put(gathered)
    finally:
        dist.destroy_process_group()


@pytest.mark.timeout(120)
def test_two_gloo_ranks_simulate_their_shards_like_one_process():
    import sys
    from pathlib import Path

    sys.path.insert(0, str(Path(__file__).resolve().parent))
    from oracle import Oracle

    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    ps = [ctx.Process(target=_simulate_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    gathered = q.get(timeout=100)
    for p in ps:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert all(g for g in gathered), "both ranks should own cloths"
    merged = {k: v for g in gathered for k, v in g.items()}
    wl = W.batched(12, frames=2, seed=5, lo=6, hi=14)
    assert sorted(merged) == list(range(len(wl.cloths)))
    for id_, spec in enumerate(wl.cloths):
        o = Oracle()
        W.build_plain(spec, o)
        for _ in range(wl.frames):
            o.simulate(wl.frame_dt, wl.substeps, wl.iterations, wl.relaxation, wl.friction,
                       wl.collision_margin, spec.particle_diameter())
        assert merged[id_] == o.positions().tobytes(), f"cloth {id_}"


@pytest.mark.timeout(120)
def test_two_gloo_ranks_shard_cloths_disjointly_and_aggregate():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    ps = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    gathered, tmax, work, total = q.get(timeout=100)
    for p in ps:
        p.join(timeout=60)
        assert p.exitcode == 0
    a, b = map(set, gathered)
    assert not (a & b) and a | b == set(range(64))
    assert tmax == 2.0 and work == total


def test_partition_balances_cost():
    rng = np.random.default_rng(0)
    costs = list(rng.integers(256, 65536, 512))
    parts = W.partition_cloths(costs, 8)
    loads = [sum(costs[i] for i in p) for p in parts]
    assert sorted(i for p in parts for i in p) == list(range(512))
    assert max(loads) / (sum(costs) / 8) < 1.01
    assert W.partition_cloths(costs, 8) == parts  # deterministic: every rank agrees
