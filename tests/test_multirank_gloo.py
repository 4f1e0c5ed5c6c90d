"""The benchmark's multi-rank path (independent replicas, max-over-ranks
timing) on two gloo ranks on the CPU."""
import os
import socket

import torch.distributed as dist
import torch.multiprocessing as mp


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    ws, r, _ = bench._dist()
    assert ws == world and r == rank
    t = bench.max_over_ranks(10.0 + rank)     # slowest rank wins
    out[rank] = t
    dist.barrier()
    dist.destroy_process_group()


def test_max_over_two_gloo_ranks():
    port = _free_port()
    out = mp.get_context("spawn").Manager().dict()
    mp.spawn(_worker, args=(2, port, out), nprocs=2, join=True)
    assert dict(out) == {0: 11.0, 1: 11.0}


def test_max_over_ranks_without_a_group():
    import bench
    assert bench.max_over_ranks(3.5) == 3.5
