"""Multi-rank (replica) logic of bench.py on CPU with gloo, world size 2: every
rank reports the slowest rank's step time and the whole-job rate counts the work
of all ranks."""

import os
import socket

import pytest
import torch.multiprocessing as mp


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, out):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    ms = bench.max_over_ranks(10.0 + 5.0 * rank, device="cpu")
    out[rank] = (ms, bench.job_rate(288, world, ms))
    dist.destroy_process_group()


def test_replica_timing_world2():
    pytest.importorskip("torch.distributed")
    world = 2
    port = _free_port()
    with mp.get_context("spawn").Manager() as mgr:
        out = mgr.dict()
        mp.spawn(_worker, args=(world, port, out), nprocs=world, join=True)
        res = dict(out)
    assert res[0][0] == res[1][0] == 15.0
    assert res[0][1] == pytest.approx(288 * 2 / 0.015)
