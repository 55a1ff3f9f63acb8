"""The multi-GPU form of the benchmark runs independent replicas: its timing
takes the maximum over ranks and its throughput adds the ranks' work. The
reduction is checked here with two gloo ranks on the CPU."""
import os
import socket

import pytest
import torch.multiprocessing as mp

import bench


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank(rank, world, port, out):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    t = bench.max_over_ranks(10.0 + rank, world, "cpu")
    out[rank] = (t, bench.replica_throughput(1000, world, t))
    dist.barrier()
    dist.destroy_process_group()


def test_replica_timing_is_the_max_over_ranks():
    world = 2
    with mp.Manager() as m:
        out = m.dict()
        mp.spawn(_rank, args=(world, _free_port(), out), nprocs=world, join=True)
        res = dict(out)
    assert res[0] == res[1] == (11.0, 2000 / 11.0)


def test_single_rank_needs_no_process_group():
    assert bench.max_over_ranks(3.5, 1) == 3.5
    assert bench.replica_throughput(10, 1, 2.0) == pytest.approx(5.0)
