"""The N>1 bench path (one rank per GPU, independent replicas) on the CPU: two gloo ranks check the
job-time reduction (max over ranks, no data-path collective) and the whole-job value, and that the
reference arm does its work on rank 0 only."""
import json
import os
import socket
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
torch = pytest.importorskip("torch")

WORKER = r"""
import os, sys, json
sys.path.insert(0, sys.argv[1])
import torch.distributed as dist
import bench
dist.init_process_group("gloo", init_method="env://")
rank, world, local = bench.dist_info()
t = bench.replica_step_time(0.5 + rank)            # rank r takes 0.5 + r seconds
v = bench.job_value(1000.0, world, t)
print(json.dumps({"rank": rank, "world": world, "t": t, "v": v}))
dist.destroy_process_group()
"""


def free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_two_gloo_replicas_reduce_the_job_time():
    port = free_port()
    procs = []
    for r in range(2):
        env = dict(os.environ, RANK=str(r), WORLD_SIZE="2", LOCAL_RANK=str(r), MASTER_ADDR="127.0.0.1",
                   MASTER_PORT=str(port))
        procs.append(subprocess.Popen([sys.executable, "-c", WORKER, ROOT], env=env, stdout=subprocess.PIPE,
                                      stderr=subprocess.PIPE, text=True))
    outs = []
    for p in procs:
        o, e = p.communicate(timeout=120)
        assert p.returncode == 0, e
        outs.append(json.loads(o.strip().splitlines()[-1]))
    for o in outs:
        assert o["world"] == 2
        assert o["t"] == 1.5                     # the slowest replica sets the job's step time
        assert o["v"] == pytest.approx(2 * 1000.0 / 1.5)


def test_reference_arm_runs_on_rank_zero_only():
    env = dict(os.environ, RANK="1", WORLD_SIZE="2", LOCAL_RANK="1")
    out = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--steps", "1",
                          "--warmup", "3"], env=env, capture_output=True, text=True, timeout=120)
    assert out.returncode == 0, out.stderr
    assert out.stdout.strip() == ""


def test_reference_arm_times_complete_solves():
    """The reference arm runs complete oracle solves of the workload (here the E=8^3 Jacobi-PCG one) with the
    oracle's own iteration count, and reports the number of solves it ran."""
    with open(os.path.join(ROOT, "tests", "golden", "config_parity.json")) as f:
        c0 = json.load(f)["c0"]
    env = dict(os.environ, RANK="0", WORLD_SIZE="1", LOCAL_RANK="0", NRSG_REF_BUDGET_S="30")
    out = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--workload",
                          "kershaw8-n7-jacobi", "--steps", "2", "--warmup", "3"], env=env, capture_output=True,
                         text=True, timeout=300)
    assert out.returncode == 0, out.stderr
    line = json.loads(out.stdout.strip().splitlines()[-1])
    assert line["impl"] == "reference" and line["config"]["iterations"] == c0["iterations"]
    assert 1 <= line["steps"] <= 2 and line["warmup"] == 0
    assert line["value"] == pytest.approx(8 ** 3 * 7 ** 3 / (line["ms_per_step"] / 1e3))
    assert line["cpu_baseline"]["kind"] == "port" and line["cpu_baseline"]["cores"] >= 1
