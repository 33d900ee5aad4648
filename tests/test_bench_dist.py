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


def test_reference_arm_prints_the_contract_line():
    """bench.py --impl reference on the host cores: one JSON line with the
    contract's keys, the warm-up it ran, an e2e object without copies, and
    the product library not loaded (the arm times the oracle alone)."""
    import json
    import subprocess
    code = ("import runpy, sys; sys.argv = ['bench.py', '--impl', 'reference', '--steps', '1',"
            " '--warmup', '3']; runpy.run_path('bench.py', run_name='__main__');"
            " print('LOADED', sorted(m for m in sys.modules if m.startswith('shear_nnf_gb300')))")
    r = subprocess.run([sys.executable, "-c", code], cwd=ROOT, capture_output=True, text=True,
                       timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = r.stdout.strip().splitlines()
    d = json.loads(lines[-2])
    for k in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step",
              "higher_is_better", "scaling", "vs_baseline", "dtype", "data", "config",
              "cpu_baseline", "e2e"):
        assert k in d, k
    assert d["impl"] == "reference" and d["warmup"] == 3 and d["value"] > 0
    assert "after 3 warm-up steps" in d["cpu_baseline"]["sample"]
    assert d["e2e"]["h2d_bytes_per_step"] == 0 and d["e2e"]["value"] == d["value"]
    assert lines[-1] == "LOADED []"
