"""The N>1 path of bench.py on CPU: replicas (one per GPU) with no data-path
collective, timed by the slowest rank. Two gloo ranks exercise the max over
ranks and the whole-job value; the reference arm's other ranks exit 0 without
work or output."""
import os
import socket
import subprocess
import sys
from pathlib import Path

import pytest
import torch.multiprocessing as mp

ROOT = Path(__file__).resolve().parents[1]


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    import torch.distributed as dist
    sys.path.insert(0, str(ROOT))
    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        local_ms = 10.0 + 5.0 * rank  # rank 1 is the slower replica
        slowest = bench.max_over_ranks(local_ms, dist, device="cpu")
        out[rank] = (slowest, bench.replica_value(world, 4.0e12, 3, slowest * 1e-3))
    finally:
        dist.destroy_process_group()


def test_two_replicas_timed_by_the_slowest():
    world = 2
    with mp.Manager() as m:
        out = m.dict()
        mp.start_processes(_rank, args=(world, _free_port(), out), nprocs=world, join=True,
                           start_method="spawn")
        res = dict(out)
    assert res[0] == res[1]  # every rank holds the job's figure
    slowest, value = res[0]
    assert slowest == 15.0
    assert value == pytest.approx(world * 4.0e12 * 3 / 0.015)


def test_reference_arm_other_ranks_exit_quietly():
    env = dict(os.environ, WORLD_SIZE="2", RANK="1", LOCAL_RANK="1")
    r = subprocess.run([sys.executable, str(ROOT / "bench.py"), "--impl", "reference", "--gpus", "2",
                        "--steps", "1", "--warmup", "1"], env=env, capture_output=True, text=True,
                       timeout=120)
    assert r.returncode == 0, r.stderr
    assert r.stdout.strip() == ""


def test_reference_arm_line():
    """The reference arm (the CPU restatement of the reference's grid loop on the
    host cores) prints one JSON line on the gb300 arm's metric, unit and config,
    with its cpu_baseline and a host-only e2e."""
    import json
    env = dict(os.environ, WORLD_SIZE="1", RANK="0")
    r = subprocess.run([sys.executable, str(ROOT / "bench.py"), "--impl", "reference", "--steps", "1",
                        "--warmup", "0"], env=env, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference"
    assert d["metric"] == "energy-grid pair evals/s" and d["unit"] == "pair evals/s"
    assert d["higher_is_better"] is True and d["value"] > 0
    assert d["cpu_baseline"]["value"] == d["value"] and d["cpu_baseline"]["cores"] >= 1
    assert d["e2e"]["h2d_bytes_per_step"] == 0 and d["e2e"]["d2h_bytes_per_step"] == 0
    assert d["config"]["workload"].startswith("framework energy grid")
