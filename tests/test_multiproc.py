"""The N > 1 path of bench.py on CPU ranks (gloo, world size 2).

Each rank runs an independent replica of the step ("replicas only": the
path's single shared exchange is inside one GPU), so the only cross-rank work
is the barrier around the timed region, the MAX of the per-rank times and the
SUM of the cells processed. Rank 1 reports a longer time and a different
cell count; every rank must see the maximum and the total.
"""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist
import torch.multiprocessing as mp


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        bench.barrier(dist)
        ms = 10.0 + 5.0 * rank            # rank 1 is the slower replica
        cells = 1000.0 * (rank + 1)
        out[rank] = (bench.reduce_max(dist, ms), bench.reduce_sum(dist, cells))
        bench.barrier(dist)
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_reduce_time_and_work():
    world = 2
    port = _free_port()
    with mp.Manager() as m:
        out = m.dict()
        mp.spawn(_rank_main, args=(world, port, out), nprocs=world, join=True)
        res = dict(out)
    assert res[0] == res[1] == (15.0, 3000.0)
