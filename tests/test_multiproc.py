"""Multi-rank bench logic on CPU (gloo, world size 2): each rank transforms
its own batch; the job time is the slowest rank's and the throughput counts
every rank's transforms.  No GPU is used."""
import os
import socket
import sys

import pytest
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, ws, port, out):
    sys.path.insert(0, ROOT)
    import torch.distributed as dist
    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(ws))
    dist.init_process_group("gloo", rank=rank, world_size=ws)
    ms, gflops = bench.aggregate(10.0 * (rank + 1), ws, 1e9, "cpu")
    out[rank] = (ms, gflops)
    dist.barrier()
    dist.destroy_process_group()


def test_two_rank_aggregate_max_time_and_total_work():
    ws = 2
    port = _free_port()
    with mp.get_context("spawn").Manager() as m:   # no fork of a process that may hold threads
        out = m.dict()
        mp.spawn(_worker, args=(ws, port, out), nprocs=ws, join=True)
        res = dict(out)
    for r in range(ws):
        ms, gflops = res[r]
        assert ms == 20.0                      # slowest rank
        assert abs(gflops - 2 * 1e9 / 20e-3 / 1e9) < 1e-9   # both ranks' work over that time
