"""The replica path of bench.py (one process per GPU, no collective on the data path) on CPU:
two gloo ranks check the max-over-ranks timing, the per-rank seed sets and that only rank 0 runs
the reference arm. The GPU legs themselves are exercised by the gpu tests."""
import os
import sys

import pytest
import torch.distributed as dist
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _rank(rank, world, port, out):
    sys.path.insert(0, ROOT)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench

    slowest = bench.max_over_ranks(10.0 + rank, world)
    bench.barrier(world)
    mine = bench.seeds(5, rank)

    class Args:
        log_vars, steps, warmup = 19, 1, 0

    bench.reference_arm(Args(), rank if rank else 1, world)  # a non-zero rank returns at once
    out[rank] = (slowest, [s.hex() for s in mine])
    dist.destroy_process_group()


def test_two_gloo_ranks():
    port = 29500 + (os.getpid() % 1000)
    with mp.Manager() as m:
        out = m.dict()
        mp.spawn(_rank, args=(2, port, out), nprocs=2, join=True)
        res = dict(out)
    assert res[0][0] == res[1][0] == 11.0
    assert not set(res[0][1]) & set(res[1][1])  # every rank proves its own seeds
    assert len(set(res[0][1])) == 5
