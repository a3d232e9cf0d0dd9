"""The N > 1 path of bench.py on the CPU: replicas only, no data-path collective.

- Two gloo ranks reduce their timings with bench.max_over_ranks (the same call the GPU run makes over
  nccl), and bench.replica_throughput turns the slowest rank's time into the whole-job rate.
- Under torchrun with two processes, the reference arm prints exactly one JSON line from rank 0; the
  other rank exits 0 without output.
"""
import json
import os
import socket
import subprocess
import sys

import pytest

from conftest import ROOT

pytest.importorskip("torch")


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


RANK_SCRIPT = r"""
import json, os, sys
sys.path.insert(0, sys.argv[1])
import torch.distributed as dist
import bench
dist.init_process_group("gloo", init_method="env://")
rank = dist.get_rank()
local_ms = 100.0 + 25.0 * rank              # rank 1 is the slower one
m = bench.max_over_ranks(local_ms)
v = bench.replica_throughput(1000, dist.get_world_size(), 3, m)
dist.barrier()
dist.destroy_process_group()
print(json.dumps({"rank": rank, "max_ms": m, "value": v}))
"""


def test_two_gloo_ranks_take_the_slowest_time():
    port = _free_port()
    procs = []
    for rank in range(2):
        env = dict(os.environ, RANK=str(rank), WORLD_SIZE="2", LOCAL_RANK=str(rank), MASTER_ADDR="127.0.0.1",
                   MASTER_PORT=str(port))
        procs.append(subprocess.Popen([sys.executable, "-c", RANK_SCRIPT, ROOT], env=env, stdout=subprocess.PIPE,
                                      stderr=subprocess.PIPE, text=True))
    outs = []
    for p in procs:
        out, err = p.communicate(timeout=120)
        assert p.returncode == 0, err[-2000:]
        outs.append(json.loads(out.strip().splitlines()[-1]))
    for o in outs:
        assert o["max_ms"] == 125.0
        assert o["value"] == pytest.approx(1000 * 2 * 3 / 0.125)


def test_single_process_needs_no_group():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.max_over_ranks(42.0) == 42.0
    assert bench.replica_throughput(10, 1, 2, 1000.0) == pytest.approx(20.0)


def test_reference_arm_under_torchrun_prints_once_from_rank_0():
    port = _free_port()
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(port), os.path.join(ROOT, "bench.py"),
           "--impl", "reference", "--workload", "air5-4096", "--gpus", "2", "--steps", "1", "--warmup", "0",
           "--cpu-seconds", "1"]
    r = subprocess.run(cmd, cwd=ROOT, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1, r.stdout
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["n_gpus"] == 2 and d["value"] > 0


def test_lane_stats_summary():
    sys.path.insert(0, ROOT)
    import bench
    import numpy as np
    s = np.zeros(24)
    s[2], s[3] = 10, 300          # rate constants: 10 warp executions, 30 lanes each
    s[17], s[18] = 750, 250       # cycles: rate constants 75%, right-hand side 25%
    d = bench.lane_stats_summary(s)
    assert d["rate constants"]["warp_executions"] == 10 and d["rate constants"]["active_lanes"] == 30.0
    assert d["rate constants"]["time_share"] == 0.75 and d["right-hand side"]["time_share"] == 0.25
    assert "time_share" not in bench.lane_stats_summary(np.zeros(24))["iteration"]
