"""The serving workload's request stream (host side, no GPU): seeded and reproducible, the
stated mix of graph kinds, n log-uniform in [20, 400], k in {1, 2, 3}, about 10 % of requests
with visibility period p in [2, 4], connected graphs, Poisson arrivals at the stated rate."""
import numpy as np

from copsandrobbers_gb300 import graphs as G
from copsandrobbers_gb300 import native as N
from copsandrobbers_gb300.serving import request_stream


def test_stream_is_seeded():
    a = request_stream(60, 45.0, seed=3)
    b = request_stream(60, 45.0, seed=3)
    assert [(r.kind, r.k, r.p, r.graph.n, r.arrival_s) for r in a] == \
           [(r.kind, r.k, r.p, r.graph.n, r.arrival_s) for r in b]
    assert all(np.array_equal(x.graph.adj, y.graph.adj) for x, y in zip(a, b))


def test_stream_mix():
    reqs = request_stream(600, 45.0, seed=12, n_hi=80)
    kinds = {r.kind for r in reqs}
    assert kinds == {"regular4", "er4", "delaunay"}
    assert {r.k for r in reqs} == {1, 2, 3}
    ps = np.array([r.p for r in reqs])
    assert set(ps[ps > 1]) <= {2, 3, 4}
    assert 0.05 < np.mean(ps > 1) < 0.15
    # about half the limited-visibility requests use the v2 rules, with k <= 2; p = 1 is v1
    v2 = [r for r in reqs if r.rules == N.CR_RULES_V2]
    assert all(1 < r.p <= 3 and r.k <= 2 and r.graph.n <= 201 for r in v2)
    assert 0.25 < len(v2) / max(1, int((ps > 1).sum())) < 0.75
    ns = np.array([r.graph.n for r in reqs])
    assert ns.min() >= 20 and ns.max() <= 81          # 4-regular graphs round n up to even
    for r in reqs[:100]:
        assert G.is_connected(r.graph.adj)
        if r.kind == "regular4":
            assert (r.graph.adj.sum(axis=1) == 4).all()


def test_poisson_arrivals_at_the_rate():
    reqs = request_stream(4000, 45.0, seed=1, n_hi=30)
    t = np.array([r.arrival_s for r in reqs])
    assert t[0] == 0.0 and np.all(np.diff(t) >= 0)
    rate = (len(t) - 1) / t[-1]
    assert 42.0 < rate < 48.0
