"""CPU, two gloo ranks: the multi-GPU host logic of the bench.  Cloths are independent,
so ranks shard by cloth with no collective on the data path; the only collectives are
the timing max and the barrier around the timed region."""
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
