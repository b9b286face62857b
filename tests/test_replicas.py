"""Multi-GPU host logic on CPU: the bench's N-replica aggregation over a
world-size-2 gloo process group (the engine runs one grid per GPU with no
collective on the data path; only the timing is reduced across ranks)."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world))
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        # rank r took 10 * (r + 1) ms for 5 steps of a 1000-cell grid
        out[rank] = bench.replica_throughput(10.0 * (rank + 1), 1000, 5, dist, "cpu")
        dist.barrier()
    finally:
        dist.destroy_process_group()


def test_replica_throughput_takes_the_slowest_rank_and_counts_every_rank():
    world = 2
    with mp.get_context("spawn").Manager() as m:  # no fork of a multi-threaded process
        out = m.dict()
        mp.spawn(_rank, args=(world, _free_port(), out), nprocs=world, join=True)
        res = dict(out)
    for r in range(world):
        ms, value = res[r]
        assert ms == 20.0
        assert value == pytest.approx(1000 * 5 * world / 0.020 / 1e9)


def test_single_replica():
    import bench
    assert bench.replica_throughput(8.0, 100, 4) == (8.0, 100 * 4 / 0.008 / 1e9)
