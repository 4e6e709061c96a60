"""The multi-rank path of bench.py on CPU (gloo, world size 2).

The loop-cluster sweep does not shard: with N ranks every rank runs an independent replica chain,
and rank 0 reports the aggregate (value = all ranks' sweeps x sites over the slowest rank's time).
These tests run that plumbing without a GPU:
* the rank reductions bench.py uses (max of the timings, sum of the work) over two gloo ranks;
* bench.py --impl reference under torchrun with two ranks: rank 0 alone times the CPU baseline
  and prints exactly one JSON line; rank 1 exits 0 without work.
"""
import json
import os
import socket
import subprocess
import sys

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _reduce_worker(rank, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), WORLD_SIZE="2",
                      RANK=str(rank), LOCAL_RANK=str(rank))
    sys.path.insert(0, REPO)
    import bench
    ws, r, _ = bench._rank_info()
    dist = bench._dist_init(ws)
    mx = bench._reduce_max(dist, 10.0 + r)       # timings: the slowest rank counts
    sm = bench._reduce_sum(dist, 100.0 * (r + 1))  # work: every rank's sweeps x sites
    bench._barrier(dist)
    dist.destroy_process_group()
    q.put((r, mx, sm))


def test_rank_reductions_over_two_gloo_ranks():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    ps = [ctx.Process(target=_reduce_worker, args=(r, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    for p in ps:
        p.join(120)
        assert p.exitcode == 0
    got = sorted(q.get(timeout=10) for _ in range(2))
    assert got == [(0, 11.0, 300.0), (1, 11.0, 300.0)]


def test_reference_arm_under_torchrun_two_ranks():
    port = _free_port()
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(port), "bench.py",
           "--impl", "reference", "--gpus", "2", "--steps", "1", "--warmup", "3", "--ref-warmup", "1"]
    env = dict(os.environ, OMP_NUM_THREADS="1")
    r = subprocess.run(cmd, cwd=REPO, capture_output=True, text=True, timeout=600, env=env)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1, r.stdout
    out = json.loads(lines[0])
    assert out["impl"] == "reference" and out["n_gpus"] == 2
    assert out["value"] > 0 and out["cpu_baseline"]["kind"] == "port"
    assert out["e2e"]["h2d_bytes_per_step"] == 0
    assert out["steps"] == 1 and out["operators_per_s"] > 0
