"""The replica logic of bench.py (N > 1 ranks) on the CPU with gloo:
rank setup from the environment, the barrier, and the max-over-ranks timing
that makes the slowest rank set the whole job's rate."""

import os
import socket

import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, out):
    os.environ.update({"RANK": str(rank), "WORLD_SIZE": str(world), "LOCAL_RANK": str(rank),
                       "MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port)})
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    w, r, l = int(os.environ["WORLD_SIZE"]), int(os.environ["RANK"]), int(os.environ["LOCAL_RANK"])
    bench.barrier(w)
    ms = 10.0 + 5.0 * r          # rank 1 is slower
    out[r] = bench.max_over_ranks(ms, w)
    dist.destroy_process_group()


def test_two_gloo_ranks_take_the_slowest_time():
    world = 2
    port = _free_port()
    out = mp.get_context("spawn").Manager().dict()
    mp.start_processes(_worker, args=(world, port, out), nprocs=world, start_method="spawn", join=True)
    assert out[0] == out[1] == 15.0
    # the job's value counts every replica at the slowest rank's rate
    assert world * 1000.0 / out[0] == pytest.approx(133.333, rel=1e-4)


def test_single_rank_passthrough():
    import bench
    assert bench.max_over_ranks(3.5, 1) == 3.5
    bench.barrier(1)
