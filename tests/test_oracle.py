"""The oracle (CPU restatement) pinned against the reference's own outputs (golden fixtures)."""
import hashlib
import os

import numpy as np
import pytest

from conftest import case_id, load_cases, matrix_path
from copsandrobbers_gb300 import graphs as G
from oracle import oracle as O

CASES = load_cases()
# every v1 case up to 2M states and every v2 case up to 50k states (the whole CPU suite stays
# within a few minutes; the larger golden cases are checked on the GPU)
SMALL = [c for c in CASES if c["config_count"] * c["n"] * c["columns"] <= (2_000_000 if c["columns"] > 1 or
         c["solver"] == "k_cops_visibility" else 50_000)]


def sha(a) -> str:
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


@pytest.mark.parametrize("case", SMALL, ids=case_id)
def test_oracle_matches_reference(case):
    g = G.load_matrix(matrix_path(case))
    if case["solver"] == "k_cops_visibility":
        sol = O.solve_v1(g, case["k"], case["p"])
    else:
        sol = O.solve_v2(g, case["k"], case["p"])
    assert sol.base_captures == case["base_captures"]
    assert sol.pass_counts == case["pass_counts"]
    assert sha(sol.states) == case["sha_states"]
    assert sha(sol.configs.reshape(-1).astype(np.uint8)) == case["sha_configs"]
    assert sha(sol.heads) == case["sha_heads"]
    assert sha(sol.transitions) == case["sha_transitions"]
    assert ("WIN" if sol.win else "LOSS") == case["result"]
    if sol.win:
        assert ", ".join(str(x) for x in sol.start_positions()) == case["positions"]
        assert sol.capture_plies == case["capture_plies"]


def test_known_answers():
    """Petersen: 2 cops lose, 3 cops win in 1 ply from (0, 2, 6)
    (console_outputs/test_results.csv of the reference, rows for peterson)."""
    g = G.load_matrix(os.path.join(os.path.dirname(__file__), "golden", "matrices", "peterson.txt"))
    assert not O.solve_v1(g, 2, 1).win
    s3 = O.solve_v1(g, 3, 1)
    assert s3.win and s3.start_positions() == (0, 2, 6) and s3.capture_plies == 1


def test_v1_col0_equals_v2_at_p1():
    """At p=1 both rule sets describe the same game: v1's column 0 equals v2's plane."""
    for name in ("peterson", "grid9", "dodecahedron", "outerplanar8"):
        g = G.load_matrix(os.path.join(os.path.dirname(__file__), "golden", "matrices", name + ".txt"))
        for k in (1, 2):
            a = O.solve_v1(g, k, 1)
            b = O.solve_v2(g, k, 1)
            assert np.array_equal(a.states[0::2], b.states)
