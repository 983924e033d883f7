"""The oracle against the reference binaries themselves, run live on freshly generated seeded
graphs (beyond the committed fixtures): states, pass counts and verdict must be identical.
The binaries are compiled from the reference's own sources by oracle/build_ref.sh; where they
are absent (the reference tree is not present) the test is skipped."""
import os

import numpy as np
import pytest

from copsandrobbers_gb300 import graphs as G
from oracle import oracle as O

REF_OK = all(os.path.exists(os.path.join(O.REF_DIR, s)) for s in ("k_cops_visibility", "k_cops_visibility_v2"))

# (generator, n, parameter, seed, k, p, solver): sizes the reference finishes in well under a second
CASES = [("er", 30, 3.0, 501, 2, 1, "k_cops_visibility"), ("er", 22, 4.0, 502, 3, 1, "k_cops_visibility"),
         ("er", 24, 2.5, 503, 2, 2, "k_cops_visibility"), ("reg", 20, 0, 504, 2, 3, "k_cops_visibility"),
         ("del", 28, 4.5, 505, 2, 1, "k_cops_visibility"), ("del", 18, 4.5, 506, 3, 2, "k_cops_visibility"),
         ("er", 14, 3.0, 507, 1, 2, "k_cops_visibility_v2"), ("del", 12, 4.5, 508, 2, 2, "k_cops_visibility_v2"),
         ("er", 10, 2.5, 509, 2, 3, "k_cops_visibility_v2"), ("reg", 12, 0, 510, 1, 3, "k_cops_visibility_v2")]


def make(kind, n, par, seed):
    if kind == "er":
        return G.erdos_renyi(n, par, seed)
    if kind == "reg":
        return G.regular4(n, seed)
    return G.delaunay_thinned(n, seed, par)


@pytest.mark.skipif(not REF_OK, reason="reference binaries not built")
@pytest.mark.parametrize("case", CASES, ids=lambda c: f"{c[0]}{c[1]}-k{c[4]}-p{c[5]}-{'v2' if c[6].endswith('v2') else 'v1'}")
def test_oracle_equals_reference_binary(tmp_path, case):
    kind, n, par, seed, k, p, solver = case
    g = make(kind, n, par, seed)
    path = tmp_path / f"{kind}{n}_{seed}.txt"
    G.save_matrix(g, path)
    ref = O.run_reference(str(path), k, p, solver, timeout=120)
    sol = O.solve_v1(g, k, p) if solver == "k_cops_visibility" else O.solve_v2(g, k, p)
    assert ref["table"] is not None, ref["stdout"][-500:]
    assert sol.pass_counts == ref["pass_counts"]
    assert sol.base_captures == ref["base_captures"]
    assert np.array_equal(sol.states, ref["table"]["states"])
    assert ("WIN" if sol.win else "LOSS") == ref["result"]


def _sweep_case(i):
    rng = np.random.default_rng(600 + i)
    kind = ("er", "reg", "del")[i % 3]
    v2 = i % 4 == 3
    n = int(rng.integers(8, 14 if v2 else 26))
    par = float(rng.uniform(2.5, 4.5))
    k = int(rng.integers(1, 3 if v2 or n > 18 else 4))
    p = int(rng.integers(1, 4))
    return kind, n if kind != "reg" else n + n % 2, par, 700 + i, k, p, "k_cops_visibility_v2" if v2 else "k_cops_visibility"


@pytest.mark.skipif(not REF_OK, reason="reference binaries not built")
@pytest.mark.parametrize("i", range(30))
def test_oracle_equals_reference_binary_sweep(tmp_path, i):
    test_oracle_equals_reference_binary(tmp_path, _sweep_case(i))
