"""Multi-rank host logic of the benchmark on CPU ranks (gloo, world size 2):
the slowest rank's time is what every rank reports, and the whole-job value
counts every rank's vertices.  No GPU."""
import os
import socket

import pytest
import torch.distributed as dist
import torch.multiprocessing as mp


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    import sys
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    import bench
    pg = bench._init_pg(world, "gloo")
    ws, r, _ = bench._dist()
    ms = 10.0 + 5.0 * r                       # rank 1 is slower
    ms_max = bench._max_over_ranks(pg, ms)
    value = bench.replica_value(1000, ws, 100, ms_max)
    out[r] = (ws, ms_max, value)
    dist.barrier()
    dist.destroy_process_group()


def test_two_replicas_report_slowest_rank():
    port = _free_port()
    with mp.get_context("spawn").Manager() as m:
        out = m.dict()
        mp.start_processes(_worker, args=(2, port, out), nprocs=2, join=True, start_method="spawn")
        res = dict(out)
    assert res[0] == res[1]
    ws, ms_max, value = res[0]
    assert ws == 2 and ms_max == 15.0
    assert value == pytest.approx(1000 * 2 * 100 / 15e-3)
