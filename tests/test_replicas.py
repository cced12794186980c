"""bench.py --gpus N runs N independent replicas (weak scaling): every rank times
its own condensate, the job time is the maximum over ranks and the value counts
the units of all ranks.  The aggregation runs here with two gloo ranks on CPU."""
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

    import bench

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        local_ms = 10.0 + 5.0 * rank      # rank 1 is the slow one
        ms, value = bench.replica_throughput(local_ms, 1000, world)
        out[rank] = (ms, value)
    finally:
        dist.destroy_process_group()


@pytest.mark.parametrize("world", [2])
def test_replica_throughput_takes_the_slowest_rank(world):
    port = _free_port()
    ctx = mp.get_context("spawn")
    with ctx.Manager() as m:
        out = m.dict()
        mp.start_processes(_rank, args=(world, port, out), nprocs=world, join=True, start_method="spawn")
        res = dict(out)
    slow = 10.0 + 5.0 * (world - 1)
    for r in range(world):
        ms, value = res[r]
        assert ms == slow
        assert value == pytest.approx(world * 1000 / (slow * 1e-3))


def test_replica_throughput_single_rank():
    import bench

    ms, value = bench.replica_throughput(4.0, 200, 1)
    assert ms == 4.0 and value == pytest.approx(5e4)
