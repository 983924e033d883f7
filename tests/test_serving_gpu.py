"""Serving: requests solved concurrently by the server give the same result as alone; the
footprint budget admits requests only while memory is left; tables stay resident."""
import numpy as np
import pytest

from copsandrobbers_gb300 import graphs as G
from copsandrobbers_gb300 import native as N
from copsandrobbers_gb300.serving import Server, request_stream, run_stream
from copsandrobbers_gb300.solver import Solver, footprint, solver_digest

pytestmark = pytest.mark.gpu


def alone(ctx, g, k, p, rules=N.CR_RULES_V1):
    with Solver(ctx, g, k, p, rules) as s:
        s.init()
        counts = s.run()
        v = s.verdict()
        return solver_digest(s), N.pass_hash(counts), v


def test_mix_equals_alone(gpu_ctx):
    reqs = request_stream(40, rate_per_s=1e6, seed=3, n_lo=12, n_hi=60)
    with Server(0, 0, workers=8) as srv:
        out = run_stream(srv, reqs, release=True)
        assert out["stats"]["max_running"] >= 2          # solves overlapped on the device
    for r, res in zip(reqs, out["results"]):
        dg, ph, v = alone(gpu_ctx, r.graph, r.k, r.p, r.rules)
        assert res["status"] == 0
        assert res["digest"] == dg and res["pass_hash"] == ph
        assert bool(res["win"]) == v.win and res["best_config"] == v.best_config


def test_mix_with_limited_visibility_equals_alone(gpu_ctx):
    # half the requests with a visibility period, half of those under the v2 rules
    reqs = request_stream(48, rate_per_s=1e6, seed=5, n_lo=10, n_hi=40, p_share=0.5)
    assert sum(r.rules == N.CR_RULES_V2 for r in reqs) >= 5
    with Server(0, 0, workers=8) as srv:
        out = run_stream(srv, reqs, release=False)
        # a resident table read back after the mix equals the same solve's table alone
        for i, (r, res) in enumerate(zip(reqs, out["results"])):
            if r.rules == N.CR_RULES_V2:
                tab = srv.read_states(out["ids"][i], int(res["states"]))
                with Solver(gpu_ctx, r.graph, r.k, r.p, r.rules) as s:
                    s.init()
                    s.run()
                    assert np.array_equal(tab, s.states())
                break
        for i in out["ids"]:
            srv.release(i)
    for r, res in zip(reqs, out["results"]):
        dg, ph, v = alone(gpu_ctx, r.graph, r.k, r.p, r.rules)
        assert res["status"] == 0
        assert res["digest"] == dg and res["pass_hash"] == ph
        assert bool(res["win"]) == v.win and res["best_config"] == v.best_config


def test_budget_admission_and_residency(gpu_ctx):
    g = G.regular4(48, 5)
    fp = footprint(48, 3, 1)
    with Server(0, int(fp * 2.5), workers=4) as srv:   # room for two resident tables
        ids = [srv.submit(g, 3, 1) for _ in range(4)]
        first = [srv.poll(i, wait_ms=-1) for i in ids[:2]]
        assert all(f is not None and f["status"] == 0 for f in first)
        # the other two wait: both earlier tables are resident and hold the budget
        assert srv.poll(ids[2], wait_ms=200) is None
        st = srv.stats()
        assert st["memory_in_use"] <= st["memory_budget"] and st["queued"] + st["running"] >= 1
        tab = srv.read_states(ids[0], int(first[0]["states"]))
        assert N.table_digest(tab) == first[0]["digest"]
        srv.release(ids[0])
        srv.release(ids[1])
        rest = [srv.poll(i, wait_ms=-1) for i in ids[2:]]
        assert all(r["digest"] == first[0]["digest"] for r in rest)


def test_oversized_request_refused():
    with Server(0, 1 << 20, workers=1) as srv:
        with pytest.raises(N.CrGpuError) as e:
            srv.submit(G.regular4(64, 1), 3, 1)
        assert e.value.code == 2


def test_concurrent_solves_on_several_threads_are_deterministic(gpu_ctx):
    """Solves of different sizes run at once from several host threads (each on its own
    context, as the server's workers do) give the tables and pass counts they give alone."""
    import threading

    reqs = request_stream(24, rate_per_s=1e6, seed=5, n_lo=10, n_hi=40, p_share=0.5)
    expect = [alone(gpu_ctx, r.graph, r.k, r.p, r.rules) for r in reqs]
    bad = []

    def worker(t):
        from copsandrobbers_gb300.solver import Context
        with Context(0) as ctx:
            for rep in range(3):
                for j in range(t, len(reqs), 2) if rep % 2 else range(len(reqs)):
                    r = reqs[j]
                    dg, ph, v = alone(ctx, r.graph, r.k, r.p, r.rules)
                    if (dg, ph) != expect[j][:2]:
                        bad.append((t, rep, j))

    ths = [threading.Thread(target=worker, args=(t,)) for t in range(6)]
    for th in ths:
        th.start()
    for th in ths:
        th.join()
    assert not bad, bad[:10]
