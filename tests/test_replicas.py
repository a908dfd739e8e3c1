"""bench.py --gpus N runs N independent replicas (the Dslash path has no
exchange step on one GPU per process): the job time is the slowest rank's,
the value counts every replica's sites.  Checked with two gloo ranks on the
CPU."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, results):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    assert bench.dist_env() == (rank, world, rank)
    mine = 10.0 + 2.5 * rank  # rank 1 is the slower replica
    results[rank] = bench.replica_time_max(mine, world, "cpu")
    dist.barrier()
    dist.destroy_process_group()


def test_replica_timing_takes_the_slowest_rank():
    import torch.multiprocessing as mp
    import bench
    ctx = mp.get_context("spawn")
    mgr = ctx.Manager()
    results = mgr.dict()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, results)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    assert results[0] == results[1] == 12.5
    # two replicas of 1,048,576 output sites x 20 steps in 12.5 ms
    v = bench.replica_gflops(12.5, 2, 1048576, 20)
    assert abs(v - 1320 * 1048576 * 20 * 2 / 12.5e6) < 1e-6 * v
    assert bench.replica_time_max(3.0, 1, "cpu") == 3.0
