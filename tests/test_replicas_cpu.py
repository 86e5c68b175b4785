"""Replica bookkeeping across processes (gloo, world size 2, no GPU)."""
import os

import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp

from dynamix_gb300 import replicas


def _worker(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        assert replicas.rank_info() == (rank, world, rank)
        ms = [12.5, 20.0][rank]                       # the slower rank sets the whole-job time
        worst = replicas.max_over_ranks(ms, dist)
        mine = replicas.shard(range(11), rank, world)
        got = [None] * world
        dist.all_gather_object(got, mine)
        out[rank] = (worst, replicas.whole_job_rate(10000, worst, world), sorted(sum(got, [])))
        dist.barrier()
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks():
    port = 29500 + os.getpid() % 1000
    with mp.Manager() as m:
        out = m.dict()
        mp.spawn(_worker, args=(2, port, out), nprocs=2, join=True)
        res = dict(out)
    for rank in (0, 1):
        worst, rate, items = res[rank]
        assert worst == 20.0
        assert rate == pytest.approx(2 * 10000 / 0.020)
        assert items == list(range(11))               # every item on exactly one rank


def test_single_process_defaults():
    assert replicas.max_over_ranks(3.5) == 3.5
    assert replicas.shard([1, 2, 3], 0, 1) == [1, 2, 3]
    assert replicas.whole_job_rate(10, 1000.0, 1) == 10.0
