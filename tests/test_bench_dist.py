"""The multi-rank side of bench.py on CPU (gloo, world size 2): each rank
steps its own shard (weak scaling, no data-path collective), the timed
region is the max over ranks, whole-job throughput counts every rank's
instances, and the reference arm runs on rank 0 alone."""
import json
import os
import socket
import subprocess
import sys

import pytest
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
import bench  # noqa: E402


def free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        ms = bench.max_over_ranks(10.0 * (rank + 1), world, "cpu")
        out.put((rank, ms, bench.whole_job_rate(world, 256, 100, ms)))
    finally:
        dist.destroy_process_group()


def test_timing_is_max_over_ranks_and_rate_counts_all_ranks():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [r[1] for r in res] == [20.0, 20.0]          # both ranks see the slowest rank's time
    assert res[0][2] == pytest.approx(2 * 256 * 100 / 0.020)


def test_shards_are_disjoint_and_deterministic():
    r0, s0 = bench.shard(0, 8)
    r1, s1 = bench.shard(1, 8)
    assert set(s0).isdisjoint(s1)
    assert r0 != r1
    assert bench.shard(1, 8) == (r1, s1)
    assert bench.max_over_ranks(3.5, 1, "cpu") == 3.5


def test_reference_arm_runs_on_rank_zero_only():
    env = dict(os.environ, OMP_NUM_THREADS="2")
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(free_port()), os.path.join(ROOT, "bench.py"),
           "--impl", "reference", "--gpus", "2", "--steps", "2", "--warmup", "3"]
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=600, env=env, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["n_gpus"] == 2 and d["value"] > 0
    assert d["e2e"]["h2d_bytes_per_step"] == 0 and d["cpu_baseline"]["kind"] in ("port", "reference")
