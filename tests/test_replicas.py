"""bench.py's whole-job timing over independent replicas, with two gloo ranks
on the CPU: every rank reports the slowest rank's step time and the job's
throughput (ranks x steps per second of the slowest)."""
import os
import socket

import torch
import torch.distributed as dist
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    import sys
    sys.path.insert(0, ROOT)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    ms = [2.0, 3.0][rank]
    ms_max, value = bench.replica_throughput(ms, world, "cpu")
    out[rank] = (ms_max, value)
    dist.destroy_process_group()


def test_replica_throughput_two_gloo_ranks():
    port = _free_port()
    with mp.Manager() as m:
        out = m.dict()
        mp.spawn(_rank, args=(2, port, out), nprocs=2, join=True)
        res = dict(out)
    for r in (0, 1):
        ms_max, value = res[r]
        assert ms_max == 3.0
        assert abs(value - 2 * 1000.0 / 3.0) < 1e-9


def test_single_replica_needs_no_process_group():
    import sys
    sys.path.insert(0, ROOT)
    import bench
    assert bench.replica_throughput(4.0, 1, "cpu") == (4.0, 250.0)
