"""Multi-GPU form = independent replicas (no collective on the data path): the host-side
rank logic of bench.py checked with two gloo ranks on the CPU — the max-over-ranks timing,
the barrier, and rank 0 alone printing the reference arm's line under torchrun."""

import json
import os
import socket
import subprocess
import sys

import pytest

from conftest import ROOT


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out_dir):
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), LOCAL_RANK=str(rank),
                      MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    sys.path.insert(0, ROOT)
    import bench

    w, r, _ = bench.dist_setup()
    bench.barrier(w)
    m = bench.allmax(w, 10.0 * (r + 1))   # each rank's timed total; the job's is the slowest
    with open(os.path.join(out_dir, f"rank{r}.txt"), "w") as f:
        f.write(f"{w} {m}")


def test_allmax_over_two_gloo_ranks(tmp_path):
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp

    port = _free_port()
    mp.spawn(_rank_main, args=(2, port, str(tmp_path)), nprocs=2, join=True)
    for r in range(2):
        w, m = open(tmp_path / f"rank{r}.txt").read().split()
        assert int(w) == 2 and float(m) == 20.0
    del torch


def test_reference_arm_under_torchrun_prints_once():
    pytest.importorskip("torch")
    port = _free_port()
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(port), os.path.join(ROOT, "bench.py"),
           "--impl", "reference", "--gpus", "2", "--scale", "0.002", "--steps", "1", "--warmup", "1"]
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=300, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1
    j = json.loads(lines[0])
    assert j["impl"] == "reference" and j["n_gpus"] == 2 and j["value"] > 0
