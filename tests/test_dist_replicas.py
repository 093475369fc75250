"""Replicas across ranks (the path has no exchange step): the bench's process-group plumbing with world_size 2 on
CPU over gloo.  Each rank runs its own replica; the only collectives are the timing barrier and the max-reduce of
the ranks' times, and rank 0 alone prints the JSON line."""
import json
import os
import socket
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


WORKER = r'''
import os, sys, json
sys.path.insert(0, {root!r})
import bench
d = bench.Dist()
assert d.world == 2
d.barrier()
m = d.max(float(d.rank) * 3.0 + 1.0)
with open(os.path.join({out!r}, "rank%d.json" % d.rank), "w") as f:
    f.write(json.dumps({{"rank": d.rank, "max": m}}))
d.close()
'''


def test_max_over_ranks_with_gloo(tmp_path):
    script = tmp_path / "w.py"
    script.write_text(WORKER.format(root=ROOT, out=str(tmp_path)))
    env = dict(os.environ, MASTER_ADDR="127.0.0.1", CUDA_VISIBLE_DEVICES="")
    r = subprocess.run([sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node=2",
                        "--master-addr=127.0.0.1", f"--master-port={free_port()}", str(script)],
                       capture_output=True, text=True, timeout=300, env=env, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [json.loads((tmp_path / f"rank{k}.json").read_text()) for k in (0, 1)]
    assert sorted(l["rank"] for l in lines) == [0, 1]
    assert all(l["max"] == 4.0 for l in lines)


def test_reference_arm_under_torchrun_prints_once():
    env = dict(os.environ, MASTER_ADDR="127.0.0.1", CUDA_VISIBLE_DEVICES="")
    r = subprocess.run([sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node=2",
                        "--master-addr=127.0.0.1", f"--master-port={free_port()}", "bench.py", "--impl", "reference",
                        "--gpus", "2", "--specimens", "3", "--total", "30000", "--steps", "1", "--warmup", "1"],
                       capture_output=True, text=True, timeout=600, env=env, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["n_gpus"] == 2 and d["value"] > 0
    assert d["cpu_baseline"]["kind"] == "port" and d["e2e"]["h2d_bytes_per_step"] == 0
