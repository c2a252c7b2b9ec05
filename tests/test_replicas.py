"""The multi-GPU form of the benchmark is replicas only: every rank contracts
the whole workload, the step time is the slowest rank's, and the job's rate is
N x the per-replica work over that time.  The host side of that (the max over
ranks and the aggregation) runs here as two gloo ranks on the CPU."""
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
    ms = bench.max_over_ranks(100.0 + 50.0 * rank, world, "cpu")
    out[rank] = (ms, bench.whole_job_tflops(world, 2e12, ms))
    dist.barrier()
    dist.destroy_process_group()


def test_two_replicas_take_the_slowest_time():
    world, port = 2, _free_port()
    with mp.Manager() as m:
        out = m.dict()
        mp.spawn(_rank, args=(world, port, out), nprocs=world, join=True)
        res = dict(out)
    assert res[0] == res[1]
    ms, value = res[0]
    assert ms == 150.0
    assert value == pytest.approx(2 * 2e12 / 0.150 / 1e12)


def test_single_replica_needs_no_process_group():
    import bench
    assert bench.max_over_ranks(42.0, 1, "cpu") == 42.0
    assert bench.whole_job_tflops(1, 1e12, 1000.0) == pytest.approx(1.0)
