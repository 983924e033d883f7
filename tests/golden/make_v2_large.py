"""Golden fixture of the limited-visibility workload at full size, from the oracle.

The workload (v2 rules on the seeded Delaunay-thinned graph, n=199, mean degree 4.5, k=2, p=3;
tests/golden/graphs/delaunay_n199_s2024.txt) is beyond what the reference's own v2 solver
finishes (it did not finish p=2 in 600 s), so its table is pinned by the oracle's restatement,
which is itself pinned to the reference on every v2 golden case of cases.json.  Records the
pass counts, base captures, verdict and SHA-256 of the states section in v2_large.json.

Re-run with:  python tests/golden/make_v2_large.py   (all host cores; minutes)
"""
from __future__ import annotations

import hashlib
import json
import os
import sys
import time

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from copsandrobbers_gb300 import graphs as G  # noqa: E402
from oracle import oracle as O  # noqa: E402


def main() -> None:
    rel = "graphs/delaunay_n199_s2024.txt"
    g = G.load_matrix(os.path.join(HERE, rel))
    k, p = 2, 3
    t0 = time.time()
    sol = O.solve_v2(g, k, p)
    dt = time.time() - t0
    case = {"graph": "delaunay_n199_s2024", "matrix": rel, "k": k, "p": p, "n": g.n,
            "solver": "oracle v2 restatement", "base_captures": sol.base_captures,
            "pass_counts": sol.pass_counts, "result": "WIN" if sol.best_config >= 0 else "LOSS",
            "best_config": sol.best_config,
            "sha_states": hashlib.sha256(sol.states.tobytes()).hexdigest(),
            "oracle_seconds": round(dt, 1)}
    with open(os.path.join(HERE, "v2_large.json"), "w") as f:
        json.dump({"delaunay_n199_k2_p3": case}, f, indent=1)
    print(json.dumps(case))


if __name__ == "__main__":
    main()
