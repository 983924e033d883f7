"""Perfect-game extraction on the device (cr_solver_perfect_game) against the reference
extractor's printed games and the oracle's walk."""
import json
import os

import numpy as np
import pytest

from conftest import GOLDEN
from copsandrobbers_gb300 import graphs as G
from copsandrobbers_gb300.solver import Solver, game_lines
from oracle import oracle as O

pytestmark = pytest.mark.gpu
GAMES = json.load(open(os.path.join(GOLDEN, "games.json")))


@pytest.mark.parametrize("case", GAMES, ids=lambda c: f"{c['graph']}-k{c['k']}")
def test_device_game_matches_reference_extractor(gpu_ctx, case):
    g = G.load_matrix(os.path.join(GOLDEN, "matrices", f"{case['graph']}.txt"))
    with Solver(gpu_ctx, g, case["k"], 1) as s:
        s.init()
        s.run()
        v = s.verdict()
        walk, captured = s.perfect_game()
        cfg = s.configs().reshape(-1, case["k"])
    assert captured and walk
    assert game_lines(cfg, v.best_config, v.capture_plies, walk) == case["lines"]


def test_device_game_matches_oracle_on_random_graphs(gpu_ctx):
    rng = np.random.default_rng(41)
    checked = 0
    for i in range(30):
        n = int(rng.integers(6, 20))
        g = G.erdos_renyi(n, float(rng.uniform(2, 4)), 500 + i)
        k = int(rng.integers(1, 4))
        sol = O.solve_v1(g, k, 1)
        with Solver(gpu_ctx, g, k, 1) as s:
            s.init()
            s.run()
            walk, captured = s.perfect_game()
        assert walk == O.perfect_game(sol, g)
        if sol.win:
            assert captured
            checked += 1
    assert checked >= 5


def test_game_needs_fixed_point_and_two_columns(gpu_ctx):
    from copsandrobbers_gb300 import native as N
    g = G.regular4(12, 3)
    with Solver(gpu_ctx, g, 2, 1) as s:
        s.init()
        with pytest.raises(N.CrGpuError) as e:
            s.perfect_game()
        assert e.value.code == 8
    with Solver(gpu_ctx, g, 2, 2) as s:
        s.init()
        s.run()
        with pytest.raises(N.CrGpuError) as e:
            s.perfect_game()
        assert e.value.code == 4
