"""Multi-process logic of bench.py on the CPU: two gloo ranks.

bench.py runs one process per GPU, each transforming its own replica of the
workload (no data-path collective); the only cross-rank steps are the barriers
around the timed region and the max over ranks of the step time.  These tests
run those steps with world_size 2 on the gloo backend, and the reference arm's
rank rule (only rank 0 runs and prints).
"""
import os
import socket
import subprocess
import sys

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


_WORKER = r"""
import os, sys, json
sys.path.insert(0, {repo!r})
import bench
rank, world, local = bench.rank_env()
ranks = bench.Ranks(world, "gloo", "cpu")
ranks.barrier()
# each rank reports a different step time; every rank must see the slowest
ms = 1.0 + rank
mx = ranks.max(ms)
ranks.barrier()
val = bench.aggregate_value(1000, world, mx)
print(json.dumps({{"rank": rank, "max": mx, "value": val}}))
import torch.distributed as dist
dist.destroy_process_group()
"""


def _spawn(world, code):
    port = _free_port()
    procs = []
    for r in range(world):
        env = dict(os.environ, RANK=str(r), WORLD_SIZE=str(world), LOCAL_RANK=str(r),
                   MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
        procs.append(subprocess.Popen([sys.executable, "-c", code], env=env,
                                      stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True))
    outs = []
    for p in procs:
        out, err = p.communicate(timeout=120)
        assert p.returncode == 0, err
        outs.append(out)
    return outs


def test_two_gloo_ranks_share_the_slowest_time():
    pytest.importorskip("torch.distributed")
    import json

    outs = _spawn(2, _WORKER.format(repo=REPO))
    res = [json.loads(o.strip().splitlines()[-1]) for o in outs]
    assert sorted(r["rank"] for r in res) == [0, 1]
    for r in res:
        assert r["max"] == 2.0                      # the slower rank's time
        assert r["value"] == pytest.approx(1000 * 2 / 2e-3)  # both ranks' work / max time


def test_single_rank_needs_no_process_group():
    sys.path.insert(0, REPO)
    import bench

    r = bench.Ranks(1, "gloo", "cpu")
    r.barrier()
    assert r.max(3.5) == 3.5
    assert bench.aggregate_value(10, 1, 2.0) == pytest.approx(5000.0)


def test_reference_arm_runs_on_rank_zero_only():
    env = dict(os.environ, RANK="1", WORLD_SIZE="2", LOCAL_RANK="1")
    p = subprocess.run([sys.executable, os.path.join(REPO, "bench.py"), "--impl", "reference"],
                       env=env, capture_output=True, text=True, timeout=120)
    assert p.returncode == 0
    assert p.stdout.strip() == ""
