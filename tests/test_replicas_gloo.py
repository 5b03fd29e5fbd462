"""bench.py's multi-rank path on CPU with the gloo backend, world size 2.

The hot path does not shard (one mesh per GPU, no domain decomposition), so N ranks run N
independent replicas; the only cross-rank traffic is bench.py's barrier and the max / sum
reductions of the timings and element counts.  These run here in two processes on 127.0.0.1.
The reference arm under torchrun is also run with two ranks: rank 0 alone times the CPU
implementation and prints the one JSON line, rank 1 exits without work.
"""
import json
import os
import socket
import subprocess
import sys

import pytest

from conftest import ROOT

WORKER = r"""
import json, os, sys
sys.path.insert(0, {root!r})
import bench
class A: pass
world, rank, local = bench.dist_setup(A())
bench.barrier(world)
mx = bench.allreduce_max(float(rank + 1) * 1.5, world)
sm = bench.allreduce_sum(float(10 * (rank + 1)), world)
bench.barrier(world)
print(json.dumps({{"rank": rank, "world": world, "local": local, "max": mx, "sum": sm}}), flush=True)
"""


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_replica_reductions_with_two_gloo_ranks():
    port = _free_port()
    procs = []
    for rank in range(2):
        env = dict(os.environ, RANK=str(rank), LOCAL_RANK=str(rank), WORLD_SIZE="2",
                   MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
        procs.append(subprocess.Popen([sys.executable, "-c", WORKER.format(root=ROOT)], env=env,
                                      stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True))
    outs = []
    for p in procs:
        out, err = p.communicate(timeout=180)
        assert p.returncode == 0, err[-2000:]
        outs.append(json.loads(out.strip().splitlines()[-1]))
    for rank, o in enumerate(sorted(outs, key=lambda o: o["rank"])):
        assert o["rank"] == rank and o["world"] == 2 and o["local"] == rank
        assert o["max"] == 3.0          # max over ranks of 1.5 (rank 0) and 3.0 (rank 1)
        assert o["sum"] == 30.0         # 10 + 20


@pytest.mark.slow
def test_reference_arm_under_torchrun_prints_one_line_from_rank_0():
    port = _free_port()
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(port), os.path.join(ROOT, "bench.py"),
           "--impl", "reference", "--gpus", "2", "--config", "C0", "--scale", "8", "--steps", "2",
           "--warmup", "3"]
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-3000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1, r.stdout
    line = json.loads(lines[0])
    assert line["impl"] == "reference" and line["n_gpus"] == 2 and line["value"] > 0
    assert line["cpu_baseline"]["kind"] == "port"
