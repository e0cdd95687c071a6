"""Multi-GPU contract on the CPU: the path does not shard (replicas only), so
bench.py under torchrun runs one independent replica per rank; its timing is
the slowest rank's and its throughput counts every rank's queries.  Checked
with two gloo ranks (no GPU), plus the reference arm's rank rule."""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _rank(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world))
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    ms, qps = bench.aggregate_replicas([10.0, 25.0][rank], 100, world, dist, "cpu")
    dist.barrier()
    dist.destroy_process_group()
    out.put((rank, ms, qps))


def test_replicas_take_the_slowest_rank_and_sum_queries():
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = 29500 + os.getpid() % 1000
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, ms, qps in res:
        assert ms == 25.0                       # the slowest replica's timed region
        assert qps == pytest.approx(200 / 0.025)  # 100 queries on each of 2 ranks


def test_single_rank_needs_no_process_group():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.aggregate_replicas(20.0, 50, 1) == (20.0, 2500.0)


def test_reference_arm_prints_the_contract_line():
    """`bench.py --impl reference` (no GPU) prints one JSON line with the
    metric, the CPU sample it timed and an e2e without device copies."""
    import json
    import subprocess
    env = dict(os.environ, RANK="0", WORLD_SIZE="1")
    out = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference",
                          "--workload", "db4096", "--steps", "2", "--warmup", "1"],
                         cwd=ROOT, env=env, capture_output=True, text=True, timeout=600)
    assert out.returncode == 0, out.stderr[-2000:]
    lines = [x for x in out.stdout.splitlines() if x.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["unit"] == "queries/s" and d["value"] > 0
    assert d["steps"] == 2 and d["warmup"] == 1 and d["higher_is_better"] is True
    assert d["config"]["workload"] == "db4096"
    assert d["cpu_baseline"]["kind"] == "port" and d["cpu_baseline"]["cores"] >= 1
    assert d["e2e"] == {"value": d["value"], "unit": "queries/s", "h2d_bytes_per_step": 0,
                        "d2h_bytes_per_step": 0}


def test_reference_arm_runs_on_rank_zero_only(monkeypatch):
    sys.path.insert(0, ROOT)
    import bench
    monkeypatch.setenv("RANK", "1")
    monkeypatch.setenv("WORLD_SIZE", "2")
    # rank 1 returns before touching the oracle or its arguments
    assert bench.run_reference(None) == 0
