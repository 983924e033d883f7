"""Stay-allowed rules (cops and robber may stay: the classical game of the reference's legacy
solver, legacy/src/k_cops_4.cpp): the oracle's v1 sweep with both self-edge rules on gives the
legacy solver's verdict and first winning start on the reference's matrices
(tests/golden/stay_verdicts.json, made by tests/golden/make_stay_golden.py)."""
import json
import os

import numpy as np
import pytest

from conftest import GOLDEN
from copsandrobbers_gb300 import graphs as G
from oracle import oracle as O

CASES = json.load(open(os.path.join(GOLDEN, "stay_verdicts.json")))


def first_universal_win(sol):
    n = sol.n
    col0 = sol.states.reshape(-1, n, sol.columns)[:, :, 0] & 1
    full = np.flatnonzero(col0.all(axis=1))
    return int(full[0]) if full.size else -1


@pytest.mark.parametrize("case", CASES, ids=lambda c: f"{c['graph']}-k{c['k']}")
def test_oracle_stay_rules_match_legacy_solver(case):
    g = G.load_matrix(os.path.join(GOLDEN, "matrices", f"{case['graph']}.txt"))
    sol = O.solve_v1(g, case["k"], 1, cop_stay=True, robber_stay=True)
    cid = first_universal_win(sol)
    assert (cid >= 0) == (case["result"] == "WIN")
    if cid >= 0:
        assert [int(x) for x in sol.configs[cid]] == case["start"]


LEGACY = os.path.join(os.path.dirname(GOLDEN), "..", "oracle", "_ref", "k_cops_4")


@pytest.mark.skipif(not os.path.exists(LEGACY), reason="legacy reference solver not built")
@pytest.mark.parametrize("i", range(16))
def test_oracle_stay_rules_match_legacy_solver_live(tmp_path, i):
    """The same check, live, on freshly generated seeded graphs."""
    import re
    import subprocess
    rng = np.random.default_rng(900 + i)
    n = int(rng.integers(8, 24))
    kind = i % 3
    g = (G.erdos_renyi(n, float(rng.uniform(2.0, 4.5)), 900 + i) if kind == 0 else
         G.regular4(n + n % 2, 900 + i) if kind == 1 else G.delaunay_thinned(n, 900 + i))
    k = int(rng.integers(1, 4 if g.n <= 16 else 3))
    path = tmp_path / "g.txt"
    G.save_matrix(g, path)
    out = subprocess.run([LEGACY, str(path), str(k)], capture_output=True, text=True, timeout=300).stdout
    m = re.search(r"RESULT: (WIN|LOSS)", out)
    assert m is not None, f"legacy solver printed no result:\n{out[-500:]}"
    result = m.group(1)
    pos = re.search(r"Optimal Cop Start Positions: \(([^)]*)\)", out)
    assert result == "LOSS" or pos is not None, f"legacy solver printed no start positions:\n{out[-500:]}"
    sol = O.solve_v1(g, k, 1, cop_stay=True, robber_stay=True)
    cid = first_universal_win(sol)
    assert (cid >= 0) == (result == "WIN")
    if cid >= 0:
        assert [int(x) for x in sol.configs[cid]] == [int(x) for x in pos.group(1).split(",")]


STAY_TABLES = json.load(open(os.path.join(GOLDEN, "stay_tables.json")))["cases"]


@pytest.mark.parametrize("case", [c for c in STAY_TABLES if not c.get("large")],
                         ids=lambda c: f"{c['graph']}-k{c['k']}-p{c['p']}-stay{c['cop_stay']}{c['robber_stay']}")
def test_oracle_stay_tables_match_reference(case):
    """The oracle's stay-rule sweep reproduces the reference v1 solver built with its self-edge
    switches flipped (tests/golden/stay_tables.json): pass counts, captures and the states."""
    import hashlib
    g = G.load_matrix(os.path.join(GOLDEN, case["matrix"]))
    sol = O.solve_v1(g, case["k"], case["p"], cop_stay=bool(case["cop_stay"]), robber_stay=bool(case["robber_stay"]))
    assert sol.pass_counts == case["pass_counts"]
    assert sol.base_captures == case["base_captures"]
    assert hashlib.sha256(sol.states.tobytes()).hexdigest() == case["sha_states"]
