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
