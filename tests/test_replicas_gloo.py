"""The N > 1 path of bench.py runs independent replicas (the step does not shard): every rank times
its own domain, the job time is the maximum over ranks and the job rate the sum.  Checked here with
two gloo ranks on the CPU."""
import os
import socket

import pytest
import torch.multiprocessing as mp


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, out):
    import sys
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    import torch.distributed as dist
    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    ms = 10.0 + 5.0 * rank            # rank 1 is the slowest replica
    job_ms = bench.max_over_ranks(ms, world, device="cpu")
    out[rank] = job_ms
    dist.destroy_process_group()


def test_replica_time_is_max_over_ranks():
    port = _free_port()
    mgr = mp.get_context("spawn").Manager()
    out = mgr.dict()
    mp.spawn(_worker, args=(2, port, out), nprocs=2, join=True)
    assert out[0] == pytest.approx(15.0) and out[1] == pytest.approx(15.0)
