"""Kernel forms of a v1 solve (cr_solver_set_forms): the fused first pass, push and pull cop
turns, the separable pull (k = 3) and the last column's fresh form are alternative ways to
compute the same pass.  Every mask, from all forms to a single one, gives the oracle's tables,
pass counts and verdicts (bit-exact), and the same table digest as the default on a solve
large enough to take the dense forms."""
import numpy as np
import pytest

from copsandrobbers_gb300 import graphs as G
from copsandrobbers_gb300 import native as N
from copsandrobbers_gb300.solver import Solver, solver_digest
from oracle import oracle as O

pytestmark = pytest.mark.gpu
ALL = N.CR_FORMS_ALL
MASKS = {
    "all": ALL,
    "unfused_first": ALL & ~N.CR_FORM_FUSED_FIRST,
    "general_last": ALL & ~N.CR_FORM_FRESH_LAST,
    "tuple_pull": ALL & ~N.CR_FORM_SEPARABLE,
    "push_only": ALL & ~N.CR_FORM_PULL,
    "pull_only": ALL & ~N.CR_FORM_PUSH,
    "tuple_pull_only": N.CR_FORM_PULL | N.CR_FORM_FUSED_FIRST | N.CR_FORM_FRESH_LAST,
    "push_minimal": N.CR_FORM_PUSH,
    "pull_minimal": N.CR_FORM_PULL,
}


def solve_masked(ctx, g, k, p, mask, rules=N.CR_RULES_V1):
    with Solver(ctx, g, k, p, rules) as s:
        s.set_forms(mask)
        s.init()
        counts = s.run()
        return counts, s.states(), s.verdict(), solver_digest(s)


@pytest.mark.parametrize("name", list(MASKS))
def test_every_form_matches_oracle(gpu_ctx, name):
    rng = np.random.default_rng(4242)
    for i in range(10):
        n = int(rng.integers(6, 36))
        g = G.erdos_renyi(n, float(rng.uniform(2, 4.5)), 700 + i) if i % 3 else G.regular4(n + n % 2, 700 + i)
        k = int(rng.integers(1, 4))
        p = int(rng.integers(1, 4)) if i % 2 else 1
        ref = O.solve_v1(g, k, p)
        counts, states, v, _ = solve_masked(gpu_ctx, g, k, p, MASKS[name])
        assert counts == ref.pass_counts, (name, i, n, k, p)
        assert np.array_equal(states, ref.states), (name, i, n, k, p)
        assert v.best_config == ref.best_config


@pytest.mark.parametrize("name", [m for m in MASKS if m != "all"])
def test_dense_solve_is_the_same_in_every_form(gpu_ctx, name):
    # a graph whose middle passes are dense (separable pull, fresh last column) and whose
    # first and last passes are sparse (push)
    g = G.erdos_renyi(72, 4.5, 7)
    base = solve_masked(gpu_ctx, g, 3, 1, ALL)
    got = solve_masked(gpu_ctx, g, 3, 1, MASKS[name])
    assert got[0] == base[0]
    assert got[3] == base[3]
    assert got[2].best_config == base[2].best_config


def test_forms_with_stay_rules(gpu_ctx):
    g = G.erdos_renyi(24, 3.0, 11)
    rules = N.CR_RULES_V1 | N.CR_COP_STAY | N.CR_ROBBER_STAY
    ref = O.solve_v1(g, 2, 2, cop_stay=True, robber_stay=True)
    for mask in (N.CR_FORM_PUSH, N.CR_FORM_PULL, ALL & ~N.CR_FORM_FRESH_LAST):
        counts, states, _, _ = solve_masked(gpu_ctx, g, 2, 2, mask, rules)
        assert counts == ref.pass_counts
        assert np.array_equal(states, ref.states)


def test_invalid_masks_refused(gpu_ctx):
    g = G.regular4(12, 3)
    with Solver(gpu_ctx, g, 2, 1) as s:
        for bad in (0, N.CR_FORM_FUSED_FIRST | N.CR_FORM_SEPARABLE, 0x40):
            with pytest.raises(N.CrGpuError) as e:
                s.set_forms(bad)
            assert e.value.code == 1
    with Solver(gpu_ctx, g, 2, 2, N.CR_RULES_V2) as s:
        s.set_forms(ALL)
        with pytest.raises(N.CrGpuError):
            s.set_forms(N.CR_FORM_PUSH)
