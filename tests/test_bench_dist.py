"""The N > 1 path of bench.py on CPU: replicas on world_size 2 gloo ranks (no GPU).

Each rank times its own replica; the job's time is the slowest rank's (an all-reduce MAX that
every rank receives) and the job's throughput counts the states of all ranks.  The reference
arm runs on rank 0 only; the other ranks exit at once without output."""
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _rank(rank, world, port, times, out):
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        ms = bench.max_over_ranks(times[rank], world, device="cpu")
        out.put((rank, ms, bench.replicas_value(1000, 10, world, ms)))
    finally:
        dist.destroy_process_group()


def test_max_over_ranks_gloo_world2():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    times = [12.5, 20.0]
    port = 29500 + os.getpid() % 1000
    procs = [ctx.Process(target=_rank, args=(r, 2, port, times, q)) for r in range(2)]
    for p in procs:
        p.start()
    got = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [g[0] for g in got] == [0, 1]
    for _, ms, value in got:
        assert ms == 20.0                       # every rank sees the slowest replica
        assert value == pytest.approx(1000 * 10 * 2 / 0.020)


def test_single_rank_needs_no_process_group():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.max_over_ranks(7.0, 1) == 7.0
    assert bench.replicas_value(100, 2, 1, 7.0) == pytest.approx(100 * 2 / 0.007)


def test_reference_arm_other_ranks_exit_quietly():
    env = dict(os.environ, RANK="1", WORLD_SIZE="2", LOCAL_RANK="1")
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--gpus", "2",
                        "--steps", "1", "--warmup", "0"], env=env, capture_output=True, text=True, timeout=120)
    assert r.returncode == 0
    assert r.stdout.strip() == ""


def test_reference_arm_json_line():
    """The reference arm's line (rank 0): the same metric and workload as the GPU arm, the
    reference's CPU path timed on all host cores, an e2e equal to its own value."""
    import json
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference",
                        "--steps", "1", "--warmup", "0"], capture_output=True, text=True, timeout=600,
                       env=dict(os.environ, RANK="0", WORLD_SIZE="1", LOCAL_RANK="0"))
    assert r.returncode == 0, r.stderr[-2000:]
    line = json.loads(r.stdout.strip().splitlines()[-1])
    assert line["impl"] == "reference"
    assert line["metric"] == "resolved states/s" and line["unit"] == "states/s"
    assert line["value"] > 0 and line["higher_is_better"] is True
    assert line["steps"] == 1 and line["warmup"] == 0 and line["n_gpus"] == 1
    assert "n=256" in line["config"]["workload"] and line["config"]["k"] == 3
    cb = line["cpu_baseline"]
    assert cb["value"] == line["value"] and cb["cores"] >= 1 and cb["kind"] in ("port", "reference")
    assert line["e2e"] == {"value": line["value"], "unit": "states/s", "h2d_bytes_per_step": 0,
                           "d2h_bytes_per_step": 0}
