"""The multi-GPU path of bench.py is replicas only (the force data is never
exchanged): world-size 2 over gloo on the CPU checks the plumbing that the
GPU runs use with NCCL -- the max over ranks, the whole-job value, the
barrier, and that only rank 0 of the reference arm does any work."""
import json
import os
import socket
import subprocess
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


_WORKER = r"""
import json, os, sys
sys.path.insert(0, sys.argv[1])
import bench
rank, local, world = bench.dist_setup(2, backend="gloo")
local_ms = 10.0 + 5.0 * rank              # rank 1 is the slower replica
bench.barrier(world)
value, ms = bench.replica_value(1.0e9, local_ms, world)
print(json.dumps({"rank": rank, "world": world, "ms": ms, "value": value}), flush=True)
import torch.distributed as dist
dist.destroy_process_group()
"""


def test_replica_plumbing_world2_gloo():
    port = _free_port()
    procs = []
    for r in range(2):
        env = dict(os.environ, MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(r),
                   LOCAL_RANK=str(r), WORLD_SIZE="2")
        procs.append(subprocess.Popen([sys.executable, "-c", _WORKER, str(ROOT)], env=env,
                                      stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True))
    outs = []
    for p in procs:
        out, err = p.communicate(timeout=120)
        assert p.returncode == 0, err
        outs.append(json.loads(out.strip().splitlines()[-1]))
    for o in outs:
        assert o["world"] == 2
        assert o["ms"] == 15.0                       # the slowest rank, on every rank
        assert o["value"] == pytest.approx(2 * 1.0e9 / 15e-3)


def test_reference_arm_runs_on_rank0_only():
    env = dict(os.environ, RANK="1", WORLD_SIZE="2", LOCAL_RANK="1")
    r = subprocess.run([sys.executable, str(ROOT / "bench.py"), "--impl", "reference",
                        "--gpus", "2", "--steps", "1", "--warmup", "1"],
                       env=env, capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stderr
    assert r.stdout.strip() == ""
