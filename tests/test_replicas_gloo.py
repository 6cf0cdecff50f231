"""Multi-rank replica accounting of bench.py, world size 2 over gloo on the CPU."""

import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench

    # rank 1 is the slow replica: the job time is its time
    ms, value = bench.replica_throughput(2.0 + 3.0 * rank, world, dist, device="cpu")
    out[rank] = (ms, value)
    dist.barrier()
    dist.destroy_process_group()


def test_replica_throughput_takes_max_over_ranks():
    world = 2
    mgr = mp.get_context("spawn").Manager()
    out = mgr.dict()
    mp.spawn(_worker, args=(world, _free_port(), out), nprocs=world, join=True)
    for rank in range(world):
        ms, value = out[rank]
        assert ms == 5.0
        assert abs(value - world * 1e3 / 5.0) < 1e-9


def test_single_rank_throughput():
    import bench

    assert bench.replica_throughput(4.0, 1) == (4.0, 250.0)
