"""Multi-process paths of bench.py on CPU (gloo, world size 2): the max-over-
ranks timing reduction, the instance partition of a batch with its host
gather, and the reference arm's launch contract (rank 0 prints one JSON line,
the other ranks exit 0 without output)."""
import json
import os
import socket
import subprocess
import sys

import pytest

from conftest import REPO

torch = pytest.importorskip("torch")


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, out):
    import torch.distributed as dist

    sys.path.insert(0, REPO)
    import bench

    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)
    try:
        batch = [f"scenario{i}" for i in range(7)]
        mine, idx = bench.shard(batch, rank, world)
        # each rank "solves" its shard: one summary row per instance it holds
        rows = [{"index": i, "iterations": 100 * i + rank} for i in idx]
        gathered = bench.gather_instances(rows, world)
        out[rank] = (bench.reduce_max(float(rank + 1) * 0.5, world, "cpu"),
                     bench.workload_seed("refinery-512", rank), bench.workload_seed("zipf-500kx1m", rank),
                     mine, [r["index"] for r in gathered], [r["iterations"] for r in gathered],
                     bench.reduce_sum([1.0, float(rank)], world, "cpu"))
    finally:
        dist.destroy_process_group()


def test_partition_gather_and_timing_world_size_2():
    """The batch partition: every rank builds the same batch (seed 0), takes
    instances rank, rank + 2, ...; the host gather gives every rank all rows in
    batch order; times reduce by max, byte counts by sum."""
    import torch.multiprocessing as mp

    port = _free_port()
    mgr = mp.get_context("spawn").Manager()  # no fork of this (multi-threaded) process
    out = mgr.dict()
    mp.spawn(_worker, args=(2, port, out), nprocs=2, join=True)
    assert out[0][0] == out[1][0] == 1.0
    assert out[0][1] == out[1][1] == 0 and out[0][2] == out[1][2] == 0  # one workload, built alike
    assert out[0][3] == ["scenario0", "scenario2", "scenario4", "scenario6"]
    assert out[1][3] == ["scenario1", "scenario3", "scenario5"]
    for r in (0, 1):
        assert out[r][4] == list(range(7))
        assert out[r][5] == [100 * i + (i % 2) for i in range(7)]
        assert out[r][6] == [2.0, 1.0]


def test_reference_arm_under_torchrun_world_size_2():
    port = _free_port()
    env = dict(os.environ)
    env.pop("CUDA_VISIBLE_DEVICES", None)
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(port), os.path.join(REPO, "bench.py"),
           "--impl", "reference", "--workload", "random-2kx5k", "--gpus", "2", "--steps", "1", "--warmup", "3"]
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=600, cwd=REPO, env=env)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["n_gpus"] == 2 and d["value"] > 0
    assert d["e2e"]["h2d_bytes_per_step"] == 0


def test_reference_arm_solves_an_mps_workload_to_tolerance(tmp_path):
    """`--workload mps:PATH` reads an MPS file; the reference arm solves it with
    the plain algorithm's CPU port until the relative KKT reaches the tolerance
    (or the iteration cap, flagged as a lower bound) and prints one JSON line."""
    path = tmp_path / "toy.mps"  # min -x1 - 2 x2, x1 + x2 <= 4, x1 - x2 <= -1, x >= 0
    path.write_text("NAME toy\nROWS\n N  OBJ\n L  R1\n L  R2\nCOLUMNS\n    X1  OBJ  -1.0  R1  1.0\n"
                    "    X1  R2  1.0\n    X2  OBJ  -2.0  R1  1.0\n    X2  R2  -1.0\nRHS\n    RHS  R1  4.0  R2  -1.0\n"
                    "ENDATA\n")
    r = subprocess.run([sys.executable, os.path.join(REPO, "bench.py"), "--impl", "reference", "--workload",
                        f"mps:{path}", "--steps", "2", "--warmup", "1"], capture_output=True, text=True, timeout=300,
                       cwd=REPO)
    assert r.returncode == 0, r.stderr[-2000:]
    d = json.loads([l for l in r.stdout.splitlines() if l.startswith("{")][0])
    assert d["impl"] == "reference" and d["value"] > 0 and d["iterations"] > 0
    assert d["config"]["workload"].startswith("mps:")
    assert d["reached_tol"] and max(d["rel_kkt"]) <= d["config"]["tol"]
