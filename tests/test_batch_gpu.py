"""GPU parity of the batched form: one persistent launch over many graphs gives, for every
(graph, k), the same table (digest), pass counts (hash), verdict and start as a single solve,
and the cop number is the first winning k."""
import numpy as np
import pytest

from copsandrobbers_gb300 import graphs as G
from copsandrobbers_gb300 import native as N
from copsandrobbers_gb300.solver import Solver, batch_solve, solver_digest
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def small_batch(count, seed, lo=8, hi=40):
    rng = np.random.default_rng(seed)
    out = []
    for i in range(count):
        n = int(rng.integers(lo, hi + 1))
        out.append(G.erdos_renyi(n, float(rng.uniform(3.0, 6.0)), G.sub_seed(seed, i) & 0xFFFFFFFF))
    return out


def single(ctx, g, k):
    with Solver(ctx, g, k, 1) as s:
        caps = s.init()
        counts = s.run()
        v = s.verdict()
        return {"digest": solver_digest(s), "pass_hash": N.pass_hash(counts), "passes": len(counts),
                "win": v.win, "best_config": v.best_config, "capture_plies": v.capture_plies,
                "base_captures": caps, "table": s.states()}


@pytest.mark.parametrize("threads", [0, 256, 512, 1024])
def test_batch_matches_single_solves(gpu_ctx, threads):
    graphs = small_batch(40, 7)
    out = batch_solve(gpu_ctx, graphs, kmax=3, p=1, threads=threads)
    assert out.stats.states > 0 and out.stats.ms > 0
    for gi, g in enumerate(graphs):
        cop = 0
        for k in range(1, 4):
            r = out.results[gi][k - 1]
            if cop:
                assert r["solved"] == 0
                continue
            s = single(gpu_ctx, g, k)
            assert r["solved"] == 1 and r["status"] == 0
            assert r["digest"] == s["digest"], (gi, k)
            assert r["pass_hash"] == s["pass_hash"] and r["passes"] == s["passes"]
            assert r["base_captures"] == s["base_captures"]
            assert bool(r["win"]) == s["win"] and r["best_config"] == s["best_config"]
            if s["win"]:
                assert r["capture_plies"] == s["capture_plies"]
                cop = k
        assert out.cop_numbers[gi] == cop


def test_digest_restated(gpu_ctx):
    for g in small_batch(6, 3):
        s = single(gpu_ctx, g, 2)
        assert s["digest"] == N.table_digest(s["table"])


def test_batch_against_oracle(gpu_ctx):
    graphs = small_batch(8, 11, 6, 20)
    out = batch_solve(gpu_ctx, graphs, kmax=3)
    for gi, g in enumerate(graphs):
        for k in range(1, 4):
            r = out.results[gi][k - 1]
            if not r["solved"]:
                continue
            ref = O.solve_v1(g, k, 1)
            assert r["digest"] == N.table_digest(ref.states)
            assert r["pass_hash"] == N.pass_hash(ref.pass_counts)
            assert r["best_config"] == ref.best_config


def test_batch_mixed_sizes_and_order(gpu_ctx):
    """Largest-first scheduling must not change any per-graph result."""
    graphs = small_batch(30, 5, 6, 128)[:12] + small_batch(30, 6, 6, 16)
    a = batch_solve(gpu_ctx, graphs, kmax=2, threads=256)
    b = batch_solve(gpu_ctx, list(reversed(graphs)), kmax=2, threads=256)
    for i in range(len(graphs)):
        j = len(graphs) - 1 - i
        assert a.cop_numbers[i] == b.cop_numbers[j]
        for k in range(2):
            assert a.results[i][k]["digest"] == b.results[j][k]["digest"]


def test_batch_limits(gpu_ctx):
    g = G.regular4(130, 1)
    with pytest.raises(N.CrGpuError) as e:
        batch_solve(gpu_ctx, [g], kmax=2)
    assert e.value.code == 4
    with pytest.raises(N.CrGpuError):
        batch_solve(gpu_ctx, small_batch(2, 1), kmax=4)
    with pytest.raises(N.CrGpuError):
        batch_solve(gpu_ctx, small_batch(2, 1), kmax=2, p=2)
