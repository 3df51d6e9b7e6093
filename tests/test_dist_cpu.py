"""The multi-rank path of bench.py (replicas only: barrier, max-over-ranks
timing, rank-0 reporting) on two gloo ranks on CPU."""
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


def _worker(rank, port, out):
    import sys
    os.environ.update({"MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port), "RANK": str(rank),
                       "WORLD_SIZE": "2", "LOCAL_RANK": str(rank), "AM_BENCH_GLOO": "1"})
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    import bench
    ws, r, _ = bench.dist_init()
    bench.barrier(ws)
    t = bench.max_over_ranks(ws, 1.0 + r, None)
    out[rank] = (ws, r, t)
    import torch.distributed as dist
    dist.destroy_process_group()


def test_two_rank_max_timing():
    port = _free_port()
    mgr = mp.Manager()
    out = mgr.dict()
    mp.spawn(_worker, args=(port, out), nprocs=2, join=True)
    assert out[0] == (2, 0, 2.0) and out[1] == (2, 1, 2.0)
