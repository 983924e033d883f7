"""GPU parity, v2 rules (limited visibility): the CUDA path against the reference's golden
outputs and the oracle."""
import hashlib

import numpy as np
import pytest

from conftest import case_id, load_cases, matrix_path
from copsandrobbers_gb300 import graphs as G
from copsandrobbers_gb300 import native as N
from copsandrobbers_gb300.solver import Solver, solve
from oracle import oracle as O

pytestmark = pytest.mark.gpu
V2 = [c for c in load_cases() if c["solver"] == "k_cops_visibility_v2"]


def sha(a) -> str:
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


@pytest.mark.parametrize("case", V2, ids=case_id)
def test_v2_matches_reference(gpu_ctx, case):
    g = G.load_matrix(matrix_path(case))
    r = solve(gpu_ctx, g, case["k"], case["p"], N.CR_RULES_V2)
    assert r.base_captures == case["base_captures"]
    assert r.pass_counts == case["pass_counts"]
    assert sha(r.states) == case["sha_states"]
    assert ("WIN" if r.verdict.win else "LOSS") == case["result"]
    if r.verdict.win:
        assert ", ".join(map(str, r.verdict.positions)) == case["positions"]
        assert r.verdict.capture_plies == case["capture_plies"]


@pytest.mark.parametrize("seed", range(10))
def test_v2_random_graphs_against_oracle(gpu_ctx, seed):
    rng = np.random.default_rng(100 + seed)
    n = int(rng.integers(6, 26))
    g = G.erdos_renyi(n, float(rng.uniform(2.0, 4.0)), 100 + seed)
    k = int(rng.integers(1, 3))
    p = int(rng.integers(1, 5))
    ref = O.solve_v2(g, k, p)
    r = solve(gpu_ctx, g, k, p, N.CR_RULES_V2)
    assert r.pass_counts == ref.pass_counts
    assert np.array_equal(r.states, ref.states)
    assert r.verdict.best_config == ref.best_config


def test_v2_table_file_bytes(gpu_ctx, tmp_path):
    for case in V2[:30]:
        g = G.load_matrix(matrix_path(case))
        with Solver(gpu_ctx, g, case["k"], case["p"], N.CR_RULES_V2) as s:
            s.init(); s.run()
            path = str(tmp_path / "t.bin")
            s.write_table_file(path)
        assert hashlib.sha256(open(path, "rb").read()).hexdigest() == case["sha_file"], case_id(case)


def test_v2_table_file_round_trip(gpu_ctx, tmp_path):
    """The v2 cache hit (k_cops_visibility_v2.cpp:170-182 -> CacheManager.h:78-141): a written
    v2 table file loads back into a fresh v2 solver as a solved table (same bytes and verdict);
    a file written for another solve is refused; initializeCaptures then resets the table."""
    for case in [c for c in V2 if c["graph"] in ("peterson", "grid9", "dodecahedron", "planar8")][:8]:
        g = G.load_matrix(matrix_path(case))
        path = str(tmp_path / "t2.bin")
        with Solver(gpu_ctx, g, case["k"], case["p"], N.CR_RULES_V2) as s:
            s.init(); counts = s.run()
            s.write_table_file(path)
            st, v = s.states(), s.verdict()
        with Solver(gpu_ctx, g, case["k"], case["p"], N.CR_RULES_V2) as t:
            t.load_table_file(path)
            assert np.array_equal(t.states(), st) and t.verdict() == v, case_id(case)
            t.init(); assert t.run() == counts
            assert np.array_equal(t.states(), st)
        with Solver(gpu_ctx, g, case["k"] % 2 + 1, case["p"], N.CR_RULES_V2) as u:   # another k
            with pytest.raises(N.CrGpuError) as e:
                u.load_table_file(path)
            assert e.value.code in (1, 7)
