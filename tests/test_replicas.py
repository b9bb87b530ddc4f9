"""The multi-GPU form of the benchmark is replicas only (a step does not shard: MIC(0) is globally
ordered): every rank runs its own step, and the only collectives are the host-side barrier and the
max / sum over ranks of bench.py.  These run here as world_size-2 gloo ranks on the CPU."""
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


RANK_SCRIPT = r"""
import json, os, sys
sys.path.insert(0, sys.argv[1])
import bench
ws, rank, _ = bench.dist_info()
D = bench.Dist(ws)
D.barrier()
out = {"rank": rank, "max": D.max(1.5 + rank), "sum": D.sum(10 * (rank + 1))}
D.barrier()
D.close()
print(json.dumps(out))
"""


def test_barrier_max_and_sum_over_two_gloo_ranks(tmp_path):
    script = tmp_path / "rank.py"
    script.write_text(RANK_SCRIPT)
    port = free_port()
    procs = []
    for r in range(2):
        env = dict(os.environ, RANK=str(r), LOCAL_RANK=str(r), WORLD_SIZE="2", MASTER_ADDR="127.0.0.1",
                   MASTER_PORT=str(port))
        procs.append(subprocess.Popen([sys.executable, str(script), ROOT], env=env, stdout=subprocess.PIPE,
                                      stderr=subprocess.PIPE, text=True))
    outs = [p.communicate(timeout=120) for p in procs]
    for p, (o, e) in zip(procs, outs):
        assert p.returncode == 0, e
    res = sorted((json.loads(o.strip().splitlines()[-1]) for o, _ in outs), key=lambda d: d["rank"])
    assert [d["max"] for d in res] == [2.5, 2.5]
    assert [d["sum"] for d in res] == [30.0, 30.0]


def test_reference_arm_under_torchrun_prints_once():
    """bench.py --impl reference launched like the multi-GPU bench: rank 0 alone runs and prints."""
    pytest.importorskip("torch")
    port = free_port()
    env = dict(os.environ, OMP_NUM_THREADS="2")
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes", "1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(port), os.path.join(ROOT, "bench.py"),
           "--impl", "reference", "--gpus", "2", "--steps", "1", "--warmup", "0"]
    r = subprocess.run(cmd, cwd=ROOT, env=env, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1, r.stdout
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["metric"] == "smoke steps/s" and d["value"] > 0
    assert d["e2e"]["h2d_bytes_per_step"] == 0 and d["cpu_baseline"]["kind"] == "port"
