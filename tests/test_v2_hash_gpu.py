"""GPU parity of the v2 cloud table (p >= 3): the depth-2 nodes each pass reaches are
deduplicated in a device hash table and evaluated once.  The tables must equal the oracle's
whatever the table's size: the default, a small table that is filled chunk by chunk and
overflows (its misses are evaluated directly), and no table at all."""
import numpy as np
import pytest

from copsandrobbers_gb300 import graphs as G
from copsandrobbers_gb300 import native as N
from copsandrobbers_gb300.solver import Solver
from oracle import oracle as O

pytestmark = pytest.mark.gpu

# (n, mean degree, seed, k, p): sizes the oracle's exhaustive search finishes in seconds
CASES = [(40, 3.5, 1, 2, 3), (32, 4.0, 2, 2, 3), (18, 3.0, 3, 3, 3), (16, 3.0, 4, 2, 4), (24, 2.5, 5, 1, 5)]


def run(ctx, g, k, p, slots=None):
    with Solver(ctx, g, k, p, N.CR_RULES_V2) as s:
        if slots is not None:
            s.set_v2_hash_capacity(slots)
        s.init()
        counts = s.run()
        return counts, s.states(), s.verdict(), s.v2_hash_stats()


@pytest.mark.parametrize("case", CASES, ids=lambda c: f"n{c[0]}-k{c[3]}-p{c[4]}")
def test_cloud_table_matches_oracle(gpu_ctx, case):
    n, deg, seed, k, p = case
    g = G.erdos_renyi(n, deg, 300 + seed)
    ref = O.solve_v2(g, k, p)
    counts, states, verdict, hs = run(gpu_ctx, g, k, p)
    assert counts == ref.pass_counts
    assert np.array_equal(states, ref.states)
    assert verdict.best_config == ref.best_config
    assert hs.capacity >= 1024 and hs.capacity & (hs.capacity - 1) == 0
    assert hs.fills == len(counts)              # one fill per pass: every node fits at once
    assert 0 < hs.entries <= hs.child_visits    # distinct nodes never exceed the visits


@pytest.mark.parametrize("slots", [0, 1024])
def test_cloud_table_size_does_not_change_results(gpu_ctx, slots):
    n, deg, seed, k, p = CASES[0]
    g = G.erdos_renyi(n, deg, 300 + seed)
    ref = O.solve_v2(g, k, p)
    counts, states, verdict, hs = run(gpu_ctx, g, k, p, slots)
    assert counts == ref.pass_counts
    assert np.array_equal(states, ref.states)
    assert verdict.best_config == ref.best_config
    assert hs.capacity == slots
    if slots:
        # C * n = 820 * 40 depth-1 nodes in chunks of 512: many fills per pass
        assert hs.fills == len(counts) * ((820 * 40 + 511) // 512)
    else:
        assert hs.fills == 0 and hs.entries == 0


def test_delaunay_clouds_repeat(gpu_ctx):
    """The limited-visibility workload's graph: the first pass's depth-2 children collapse to
    far fewer distinct nodes (the dedup the table exists for)."""
    import os
    path = os.path.join(os.path.dirname(__file__), "golden", "graphs", "delaunay_n199_s2024.txt")
    g = G.load_matrix(path)
    with Solver(gpu_ctx, g, 2, 3, N.CR_RULES_V2) as s:
        s.init()
        s.step()
        hs = s.v2_hash_stats()
    assert hs.fills == 1
    assert hs.child_visits > 10 * hs.entries > 0


def test_v1_has_no_cloud_table(gpu_ctx):
    g = G.erdos_renyi(12, 3.0, 7)
    with Solver(gpu_ctx, g, 2, 3, N.CR_RULES_V1) as s:
        s.set_v2_hash_capacity(4096)            # ignored: v1 rules keep no clouds
        assert s.v2_hash_stats().capacity == 0


@pytest.mark.slow
@pytest.mark.parametrize("slots", [None, 0])
def test_limited_visibility_workload_full_size(gpu_ctx, slots):
    """The limited-visibility workload itself (Delaunay-thinned n=199, k=2, p=3, 3.96 M states)
    against the oracle's table (tests/golden/v2_large.json, made by make_v2_large.py; the
    reference's own v2 solver does not finish this graph), with and without the cloud table."""
    import hashlib
    import json
    import os
    here = os.path.join(os.path.dirname(__file__), "golden")
    case = json.load(open(os.path.join(here, "v2_large.json")))["delaunay_n199_k2_p3"]
    g = G.load_matrix(os.path.join(here, case["matrix"]))
    with Solver(gpu_ctx, g, case["k"], case["p"], N.CR_RULES_V2) as s:
        if slots is not None:
            s.set_v2_hash_capacity(slots)
        assert s.init() == case["base_captures"]
        assert s.run() == case["pass_counts"]
        v = s.verdict()
        st = s.states()
    assert hashlib.sha256(st.tobytes()).hexdigest() == case["sha_states"]
    assert ("WIN" if v.win else "LOSS") == case["result"]
    assert v.best_config == case["best_config"]
