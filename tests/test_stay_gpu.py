"""Stay-allowed rules on the device (CR_COP_STAY / CR_ROBBER_STAY): tables, pass counts and
verdicts bit-exact against the oracle for every combination of the two flags."""
import numpy as np
import pytest

from copsandrobbers_gb300 import graphs as G
from copsandrobbers_gb300 import native as N
from copsandrobbers_gb300.solver import solve
from oracle import oracle as O

pytestmark = pytest.mark.gpu
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
