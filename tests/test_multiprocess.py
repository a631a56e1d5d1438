"""The multi-GPU path of bench.py (replicas: one process per GPU, no
collective on the data path) run as world-size-2 process groups on the CPU
with the gloo backend: the step time is the slowest rank's, the value counts
every rank's clouds, and the reference arm prints on rank 0 only."""
import json
import multiprocessing as mp
import os
import socket
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world), LOCAL_RANK=str(rank))
    sys.path.insert(0, ROOT)
    import torch.distributed as dist

    import bench

    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        r, w, _ = bench.dist_env()
        ms = bench.max_over_ranks(10.0 + 5.0 * r, w, "cpu")  # rank 1 is the slow one
        q.put((r, ms, bench.job_value(256, w, ms / 1e3)))
    finally:
        dist.destroy_process_group()


def test_replicas_take_the_slowest_rank_gloo():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [o[0] for o in out] == [0, 1]
    for _, ms, value in out:
        assert ms == 15.0  # both ranks see the slowest step
        assert value == pytest.approx(2 * 256 / 0.015)


def _bench(env_extra, *args):
    env = dict(os.environ, **env_extra)
    return subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), *args],
                          capture_output=True, text=True, env=env, timeout=600)


def test_reference_arm_prints_on_rank_zero_only():
    args = ("--impl", "reference", "--workload", "single-4k", "--steps", "1", "--warmup", "1")
    r1 = _bench({"RANK": "1", "WORLD_SIZE": "2", "LOCAL_RANK": "1"}, *args)
    assert r1.returncode == 0 and r1.stdout.strip() == ""
    r0 = _bench({"RANK": "0", "WORLD_SIZE": "2", "LOCAL_RANK": "0"}, *args)
    assert r0.returncode == 0, r0.stderr[-2000:]
    lines = [l for l in r0.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    line = json.loads(lines[0])
    assert line["impl"] == "reference" and line["value"] > 0
    assert line["e2e"]["h2d_bytes_per_step"] == 0 and line["cpu_baseline"]["cores"] >= 1


def test_served_reference_arm_line():
    """bench.py --impl reference --workload served: the requests of the
    replayed window timed on the host cores and served first come, first
    served, reported in the GPU served line's units."""
    env = dict(os.environ, PYTHONPATH=ROOT)
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference",
                        "--workload", "served", "--served-window", "0.0002"],
                       capture_output=True, text=True, env=env, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    line = json.loads(r.stdout.strip().splitlines()[-1])
    assert line["impl"] == "reference" and line["metric"] == "requests/sec (served)"
    assert line["config"]["requests"] == 1 and line["value"] > 0
    assert line["latency_ms"]["p50"] > 0 and line["cpu_baseline"]["cores"] == 1
