"""The multi-GPU form of the benchmark is independent replicas (no data-path
collective): ranks time their own steps and the job reports the slowest
rank's time.  Checked on CPU with two gloo ranks."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")


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
    import bench
    mine = [1.0 + rank, 10.0 - rank, 0.5 * (rank + 1)]
    got = bench.max_over_ranks(mine, world, "cpu")
    out[rank] = (got, bench.replica_throughput(world, 160, got[0]))
    dist.barrier()
    dist.destroy_process_group()


def test_max_over_ranks_two_gloo_ranks():
    import torch.multiprocessing as mp
    world = 2
    port = _free_port()
    mgr = mp.Manager()
    out = mgr.dict()
    mp.spawn(_rank, args=(world, port, out), nprocs=world, join=True)
    for r in range(world):
        got, tput = out[r]
        assert got == [2.0, 10.0, 1.0]          # the slowest rank's values
        assert tput == pytest.approx(2 * 160 / 2.0)


def test_single_rank_passthrough():
    import bench
    assert bench.max_over_ranks([3.0, 4.0], 1, "cpu") == [3.0, 4.0]
    assert bench.replica_throughput(1, 16, 0.5) == 32.0
