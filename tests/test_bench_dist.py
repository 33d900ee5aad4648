"""The multi-rank timing of bench.py (replicas, one box per rank, no data-path
collective): barrier and max over ranks, with world_size 2 over gloo."""
import os
import socket
import sys

import pytest
import torch.multiprocessing as mp

from conftest import ROOT


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank(rank, ws, port, out):
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(ws), LOCAL_RANK=str(rank),
                      MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    sys.path.insert(0, ROOT)
    import bench
    dist, r, w = bench.dist_setup()
    assert (r, w) == (rank, ws) and dist is not None
    bench.barrier(dist)
    out[rank] = bench.allmax(dist, 1.5 + 2.0 * rank)
    bench.barrier(dist)
    dist.destroy_process_group()


def test_replica_timing_takes_the_slowest_rank():
    ws = 2
    out = mp.get_context("spawn").Manager().dict()
    mp.spawn(_rank, args=(ws, _free_port(), out), nprocs=ws, join=True)
    assert dict(out) == {0: 3.5, 1: 3.5}
