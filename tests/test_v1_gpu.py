"""GPU parity, v1 rules: the CUDA path against the reference's golden outputs and the oracle."""
import hashlib

import numpy as np
import pytest

from conftest import case_id, load_cases, matrix_path
from copsandrobbers_gb300 import graphs as G
from copsandrobbers_gb300 import native as N
from copsandrobbers_gb300.solver import Solver, solve
from oracle import oracle as O

pytestmark = pytest.mark.gpu
V1 = [c for c in load_cases() if c["solver"] == "k_cops_visibility"]


def sha(a) -> str:
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


@pytest.mark.parametrize("case", V1, ids=case_id)
def test_v1_matches_reference(gpu_ctx, case):
    g = G.load_matrix(matrix_path(case))
    r = solve(gpu_ctx, g, case["k"], case["p"], N.CR_RULES_V1)
    assert r.base_captures == case["base_captures"]
    assert r.pass_counts == case["pass_counts"]
    assert sha(r.states) == case["sha_states"]
    assert ("WIN" if r.verdict.win else "LOSS") == case["result"]
    if r.verdict.win:
        assert ", ".join(map(str, r.verdict.positions)) == case["positions"]
        assert r.verdict.capture_plies == case["capture_plies"]


@pytest.mark.parametrize("seed", range(12))
def test_v1_random_graphs_against_oracle(gpu_ctx, seed):
    rng = np.random.default_rng(seed)
    n = int(rng.integers(5, 40))
    g = G.erdos_renyi(n, float(rng.uniform(2.0, 5.0)), seed)
    k = int(rng.integers(1, 4)) if n <= 24 else int(rng.integers(1, 3))
    p = int(rng.integers(1, 4))
    ref = O.solve_v1(g, k, p)
    r = solve(gpu_ctx, g, k, p, N.CR_RULES_V1)
    assert r.pass_counts == ref.pass_counts
    assert np.array_equal(r.states, ref.states)
    assert r.verdict.best_config == ref.best_config


def test_v1_phase_by_phase_equals_whole(gpu_ctx):
    g = G.load_matrix(matrix_path(next(c for c in V1 if c["graph"] == "peterson")))
    with Solver(gpu_ctx, g, 3, 1) as s:
        caps = s.init()
        counts = []
        while True:
            f = s.step()
            counts.append(f)
            if f == 0:
                break
        assert s.step() == 0          # the fixed point is sticky
        v = s.verdict()
        st = s.states()
    r = solve(gpu_ctx, g, 3, 1)
    assert caps == r.base_captures and counts == r.pass_counts
    assert np.array_equal(st, r.states) and v == r.verdict


def test_v1_reinit_gives_same_table(gpu_ctx):
    """initializeCaptures resets every column, so solving twice on one state store is identical
    (the cache-hit invariant of k_cops_visibility.cpp:92-104)."""
    g = G.erdos_renyi(30, 4.0, 5)
    with Solver(gpu_ctx, g, 2, 2) as s:
        s.init(); a = s.run(); sa = s.states()
        s.init(); b = s.run(); sb = s.states()
    assert a == b and np.array_equal(sa, sb)


def test_v1_transitions_and_configs(gpu_ctx):
    for case in [c for c in V1 if c["p"] == 1 and c["config_count"] * c["n"] < 3_000_000][:40]:
        g = G.load_matrix(matrix_path(case))
        with Solver(gpu_ctx, g, case["k"], case["p"]) as s:
            heads, data = s.transitions()
            assert sha(heads) == case["sha_heads"], case_id(case)
            assert sha(data) == case["sha_transitions"], case_id(case)
            assert sha(s.configs()) == case["sha_configs"], case_id(case)


def test_v1_table_file_bytes(gpu_ctx, tmp_path):
    for case in [c for c in V1 if c["graph"] in ("peterson", "grid9", "dodecahedron")]:
        g = G.load_matrix(matrix_path(case))
        with Solver(gpu_ctx, g, case["k"], case["p"]) as s:
            s.init(); s.run()
            path = str(tmp_path / "t.bin")
            s.write_table_file(path)
        assert hashlib.sha256(open(path, "rb").read()).hexdigest() == case["sha_file"], case_id(case)


def test_table_file_round_trip(gpu_ctx, tmp_path):
    """CacheManager::loadAuxGraph: a written table file loads back into a fresh solver as a
    solved table (same bytes, verdict and perfect game); initializeCaptures then resets it."""
    import hashlib
    from copsandrobbers_gb300.solver import Solver
    for case in [c for c in V1 if c["graph"] in ("peterson", "grid9", "dodecahedron") and c["p"] <= 2]:
        g = G.load_matrix(matrix_path(case))
        path = str(tmp_path / "t.bin")
        with Solver(gpu_ctx, g, case["k"], case["p"]) as s:
            s.init(); counts = s.run()
            s.write_table_file(path)
            st, v = s.states(), s.verdict()
            game = s.perfect_game() if case["p"] == 1 else None
        with Solver(gpu_ctx, g, case["k"], case["p"]) as t:
            t.load_table_file(path)
            assert np.array_equal(t.states(), st) and t.verdict() == v, case_id(case)
            if game is not None:
                assert t.perfect_game() == game
            assert hashlib.sha256(open(path, "rb").read()).hexdigest() == case["sha_file"]
            t.init(); assert t.run() == counts
            assert np.array_equal(t.states(), st)
        # written for another solve: refused
        with Solver(gpu_ctx, g, case["k"] % 3 + 1, case["p"]) as u:
            with pytest.raises(N.CrGpuError) as e:
                u.load_table_file(path)
            assert e.value.code in (1, 7)
