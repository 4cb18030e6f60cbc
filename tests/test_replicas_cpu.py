"""The multi-GPU mode of bench.py is replicas only (one block per rank, no
data-path collective): its only cross-rank step is the MAX of the ranks'
times.  Checked here with two gloo ranks on the CPU, and the reference arm's
rule that ranks other than 0 print nothing."""
import os
import socket
import subprocess
import sys

import pytest
import torch.distributed as dist
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    t = bench.max_over_ranks(10.0 + rank, dist, "cpu")
    out[rank] = (t, bench.replica_rate(1000, 10, world, t))
    dist.destroy_process_group()


def test_two_rank_max_and_rate():
    port = _free_port()
    out = mp.get_context("spawn").Manager().dict()  # no fork of a threaded process
    mp.spawn(_rank, args=(2, port, out), nprocs=2, join=True)
    assert out[0][0] == out[1][0] == 11.0
    assert out[0][1] == pytest.approx(2 * 1000 * 10 / 11.0 / 1e6)


def test_reference_arm_silent_off_rank_zero():
    env = dict(os.environ, RANK="1", WORLD_SIZE="2", LOCAL_RANK="1")
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference",
                        "--steps", "1", "--warmup", "0"], env=env, capture_output=True, text=True,
                       timeout=120)
    assert r.returncode == 0 and r.stdout.strip() == ""


def test_reference_arm_line_on_rank_zero():
    """rank 0 of the reference arm times the oracle on the host cores and
    prints one JSON line with the contract's keys: every requested warm-up
    iteration run, no host<->device bytes, the cpu_baseline describing the
    run itself"""
    import json
    env = dict(os.environ, RANK="0", WORLD_SIZE="1", LOCAL_RANK="0")
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference",
                        "--steps", "1", "--warmup", "3"], env=env, capture_output=True, text=True,
                       timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.strip()]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["warmup"] == 3 and d["steps"] == 1
    assert d["value"] > 0 and d["unit"] == "Mcell-residuals/s" and d["higher_is_better"] is True
    assert d["e2e"]["h2d_bytes_per_step"] == 0 and d["e2e"]["d2h_bytes_per_step"] == 0
    assert d["cpu_baseline"]["value"] == d["value"] and d["cpu_baseline"]["cores"] >= 1
    assert d["config"]["workload"].startswith("smooth bump 256x96x4")
