"""The multi-rank host logic of bench.py, as two gloo ranks on the CPU: the
barrier, max-over-ranks timing and whole-job sums, per-rank workloads that
do not overlap (replicas and served traces shard by seed), and the reference
arm running on rank 0 only."""
import json
import os
import socket
import subprocess
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent

CHILD = r"""
import json, sys, types
sys.path.insert(0, sys.argv[1])
import bench
from opensayal_gb300 import scenarios
world, rank, local = bench.dist_setup()
out = {"world": world, "rank": rank}
bench.dist_barrier(world)
out["max"] = bench.dist_max(world, 1.5 + rank)
out["sum"] = bench.dist_sum(world, 1.0 + rank)
cfgs = scenarios.batched_scenarios(6, seed=4 + 1000 * rank)
out["batched"] = [(c.width, c.height, c.projection_n, round(c.tunnel_speed, 6)) for c in cfgs]
reqs = scenarios.serving_requests(50.0, 0.5, seed=5 + 1000 * rank)
out["served"] = [(round(r.arrival, 9), r.cells, r.steps) for r in reqs]
args = types.SimpleNamespace(workload="small", steps=1, warmup=1, block=None)
out["reference_arm_none"] = rank != 0 and bench.run_reference(args, world, rank, local) is None
bench.dist_barrier(world)
import torch.distributed as dist
dist.destroy_process_group()
json.dump(out, open(sys.argv[2], "w"))
"""


def free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_two_gloo_ranks(tmp_path):
    pytest.importorskip("torch.distributed")
    port = free_port()
    procs = []
    for rank in range(2):
        env = dict(os.environ, WORLD_SIZE="2", RANK=str(rank), LOCAL_RANK=str(rank),
                   MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), CUDA_VISIBLE_DEVICES="")
        procs.append(subprocess.Popen(
            [sys.executable, "-c", CHILD, str(ROOT), str(tmp_path / f"r{rank}.json")], env=env,
            stdout=subprocess.PIPE, stderr=subprocess.STDOUT))
    for p in procs:
        out, _ = p.communicate(timeout=240)
        assert p.returncode == 0, out.decode()[-2000:]
    r0, r1 = (json.loads((tmp_path / f"r{k}.json").read_text()) for k in range(2))
    assert r0["world"] == r1["world"] == 2 and (r0["rank"], r1["rank"]) == (0, 1)
    assert r0["max"] == r1["max"] == 2.5
    assert r0["sum"] == r1["sum"] == 3.0
    assert r0["batched"] != r1["batched"]
    assert r0["served"] != r1["served"] and len(r0["served"]) > 5
    assert r1["reference_arm_none"] is True
