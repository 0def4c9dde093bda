"""Multi-GPU runs are replicas (the path does not shard: runs are independent),
so the only multi-rank logic is the whole-job aggregate of bench.py: the
slowest rank's time and the units all ranks processed.  Checked here with
two gloo ranks on the CPU (127.0.0.1)."""
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    import bench
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        ms, units = bench.whole_job(10.0 + 5.0 * rank, 1000.0 * (rank + 1), dist, "cpu")
        dist.barrier()
        out[rank] = (ms, units)
    finally:
        dist.destroy_process_group()


def test_whole_job_aggregate_two_gloo_ranks():
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp
    world, port = 2, _free_port()
    with mp.Manager() as m:
        out = m.dict()
        mp.spawn(_rank, args=(world, port, out), nprocs=world, join=True)
        res = dict(out)
    assert res[0] == res[1] == (15.0, 3000.0)


def test_whole_job_single_process_is_identity():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.whole_job(7.5, 123.0) == (7.5, 123.0)
