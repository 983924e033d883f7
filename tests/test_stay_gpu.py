"""Stay-allowed rules on the device (CR_COP_STAY / CR_ROBBER_STAY): tables, pass counts and
verdicts bit-exact against the reference v1 solver built with its self-edge switches flipped
(tests/golden/stay_tables.json, including two larger solves that take the push, separable and
fused first-pass forms), and against the oracle on random graphs for every flag combination."""
import hashlib
import json
import os

import numpy as np
import pytest

from copsandrobbers_gb300 import graphs as G
from copsandrobbers_gb300 import native as N
from copsandrobbers_gb300.solver import solve
from conftest import GOLDEN
from oracle import oracle as O

pytestmark = pytest.mark.gpu
STAY_TABLES = json.load(open(os.path.join(GOLDEN, "stay_tables.json")))["cases"]
FLAGS = [(False, False), (True, False), (False, True), (True, True)]


@pytest.mark.parametrize("cop_stay,robber_stay", FLAGS)
def test_stay_rules_match_oracle(gpu_ctx, cop_stay, robber_stay):
    rng = np.random.default_rng(7 + 2 * cop_stay + robber_stay)
    rules = N.CR_RULES_V1 | (N.CR_COP_STAY if cop_stay else 0) | (N.CR_ROBBER_STAY if robber_stay else 0)
    for i in range(12):
        n = int(rng.integers(5, 24))
        g = G.erdos_renyi(n, float(rng.uniform(1.5, 4)), 900 + i) if i % 3 else G.regular4(n + n % 2, 900 + i)
        k = int(rng.integers(1, 4))
        p = int(rng.integers(1, 3))
        ref = O.solve_v1(g, k, p, cop_stay=cop_stay, robber_stay=robber_stay)
        r = solve(gpu_ctx, g, k, p, rules)
        assert r.pass_counts == ref.pass_counts, (i, n, k, p)
        assert np.array_equal(r.states, ref.states), (i, n, k, p)
        assert r.verdict.best_config == ref.best_config


def test_stay_rules_refused_for_v2(gpu_ctx):
    with pytest.raises(N.CrGpuError) as e:
        solve(gpu_ctx, G.regular4(10, 1), 2, 2, N.CR_RULES_V2 | N.CR_COP_STAY)
    assert e.value.code == 4


@pytest.mark.parametrize("case", STAY_TABLES,
                         ids=lambda c: f"{c['graph']}-k{c['k']}-p{c['p']}-stay{c['cop_stay']}{c['robber_stay']}")
def test_stay_tables_match_reference(gpu_ctx, case):
    g = G.load_matrix(os.path.join(GOLDEN, case["matrix"]))
    rules = N.CR_RULES_V1 | (N.CR_COP_STAY if case["cop_stay"] else 0) | (N.CR_ROBBER_STAY if case["robber_stay"] else 0)
    r = solve(gpu_ctx, g, case["k"], case["p"], rules)
    assert r.pass_counts == case["pass_counts"]
    assert r.base_captures == case["base_captures"]
    assert hashlib.sha256(r.states.tobytes()).hexdigest() == case["sha_states"]
    assert r.verdict.win == (case["result"] == "WIN")
    if r.verdict.win:
        assert ",".join(str(x) for x in r.verdict.positions) == case["positions"].replace(" ", "")
        assert r.verdict.capture_plies == case["capture_plies"]
