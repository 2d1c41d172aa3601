"""The N > 1 path of bench.py on CPU: two gloo ranks, independent replicas.

Each rank reports its own time and units; the result must be the sum of the
units over the slowest rank's time, and ranks must draw different operands.
"""
import os
import socket

import pytest
import torch.multiprocessing as mp


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    import torch.distributed as dist
    from vkhel_gb300 import replicas
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    units, secs, rate = replicas.aggregate(local_seconds=1.0 + rank, local_units=100 * (rank + 1))
    out[rank] = (units, secs, rate, replicas.rank_seed(2, rank), replicas.shard(list(range(10)), rank, world))
    dist.barrier()
    dist.destroy_process_group()


def test_two_gloo_ranks_aggregate_as_independent_replicas():
    world = 2
    with mp.Manager() as m:
        out = m.dict()
        mp.spawn(_rank, args=(world, _free_port(), out), nprocs=world, join=True)
        res = dict(out)
    for rank in range(world):
        units, secs, rate, seed, part = res[rank]
        assert units == 300 and secs == 2.0 and rate == pytest.approx(150.0)
    assert res[0][3] != res[1][3]
    assert sorted(res[0][4] + res[1][4]) == list(range(10))


def test_single_rank_without_process_group():
    from vkhel_gb300 import replicas
    assert replicas.aggregate(2.0, 10) == (10, 2.0, 5.0)
