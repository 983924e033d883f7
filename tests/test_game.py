"""Perfect-game extraction (util/perfect_game_extractor.py): the oracle's restatement of the
walk, printed the reference's way, equals what the reference's own extractor printed on the
same tables (tests/golden/games.json, made by tests/golden/make_games.py)."""
import json
import os

import pytest

from conftest import GOLDEN
from copsandrobbers_gb300 import graphs as G
from copsandrobbers_gb300.solver import game_lines
from oracle import oracle as O

GAMES = json.load(open(os.path.join(GOLDEN, "games.json")))


@pytest.mark.parametrize("case", GAMES, ids=lambda c: f"{c['graph']}-k{c['k']}")
def test_oracle_walk_matches_reference_extractor(case):
    g = G.load_matrix(os.path.join(GOLDEN, "matrices", f"{case['graph']}.txt"))
    sol = O.solve_v1(g, case["k"], 1)
    walk = O.perfect_game(sol, g)
    assert sol.win == case["win"]
    if not sol.win:
        assert walk == []
        return
    assert game_lines(sol.configs, sol.best_config, sol.capture_plies, walk) == case["lines"]
