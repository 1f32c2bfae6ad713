"""`bench.py --impl reference` (the CPU oracle timed on the host, no GPU) on a small asteroid step:
one JSON line with the GPU arm's metric, unit and workload name, a `cpu_baseline` describing the run
and an `e2e` without host-device copies; under two gloo ranks only rank 0 prints it."""
import json
import os
import socket
import subprocess
import sys

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SMALL = ["--faces", "20000", "--res", "128", "--lidar", "64", "--cpu-seconds", "0.5", "--steps", "2",
         "--warmup", "3"]


def json_lines(text):
    return [json.loads(s) for s in text.splitlines() if s.startswith("{")]


def test_reference_arm_line():
    sys.path.insert(0, REPO)
    import bench
    r = subprocess.run([sys.executable, "bench.py", "--impl", "reference"] + SMALL, cwd=REPO, capture_output=True,
                       text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = json_lines(r.stdout)
    assert len(lines) == 1
    d = lines[0]
    assert d["impl"] == "reference" and d["metric"] == bench.METRIC and d["unit"] == bench.UNIT
    assert d["higher_is_better"] is True and d["n_gpus"] == 1 and d["steps"] == 2 and d["warmup"] == 3
    assert d["value"] > 0 and d["ms_per_step"] > 0
    assert d["config"]["workload"] == "asteroid-20000: render 128^2 1 spp (primary + sun shadow) + LiDAR 64^2 " \
                                      "(range + triangle id)"
    cb = d["cpu_baseline"]
    assert cb["kind"] == "port" and cb["value"] == d["value"] and cb["cores"] >= 1 and cb["sample"]
    assert d["e2e"] == {"value": d["value"], "unit": d["unit"], "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}


def test_reference_arm_two_ranks_rank0_prints():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2", "--master-addr",
           "127.0.0.1", "--master-port", str(port), "bench.py", "--impl", "reference", "--gpus", "2"] + SMALL
    env = dict(os.environ, OMP_NUM_THREADS="1")
    r = subprocess.run(cmd, cwd=REPO, capture_output=True, text=True, timeout=600, env=env)
    if r.returncode != 0 and "Address already in use" in r.stderr:
        pytest.skip("rendezvous port taken")
    assert r.returncode == 0, r.stderr[-2000:]
    lines = json_lines(r.stdout)
    assert len(lines) == 1 and lines[0]["impl"] == "reference" and lines[0]["n_gpus"] == 2
