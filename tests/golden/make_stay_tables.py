"""Golden tables of the stay-allowed rule sets, from the reference's own v1 solver.

oracle/build_ref.sh builds solvers/k_cops_visibility.cpp three more times with its two
self-edge switches (SelfEdgeCop, SelfEdgeRobber, lines 63-64) flipped: cops may stay (10),
the robber may stay (01), both (11).  This script runs those binaries on the reference's own
matrices (k <= 3, p <= 2, within a state cap) and on two larger seeded graphs whose solves take
the device's push, separable and fused-first-pass forms, and records what each printed and the
SHA-256 of the states section of the table file it wrote.

    python tests/golden/make_stay_tables.py   ->  tests/golden/stay_tables.json
(needs oracle/_ref/ built from the reference tree)
"""
from __future__ import annotations

import hashlib
import json
import math
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import oracle as O  # noqa: E402
from copsandrobbers_gb300 import graphs as G  # noqa: E402

SMALL = ["cycle5", "cycle10", "line10", "tree7", "grid9", "rooks", "planar8", "outerplanar8",
         "peterson", "robertson", "dodecahedron", "dismantleable19", "planar32", "grid36"]
STATE_CAP = 3_000_000
RULES = {"10": (1, 0), "01": (0, 1), "11": (1, 1)}
LARGE = [("regular4_n64_s777", lambda: G.regular4(64, 777), 3),
         ("er_n48_d4.5_s31", lambda: G.erdos_renyi(48, 4.5, 31), 3)]


def case(path: str, name: str, k: int, p: int, code: str) -> dict | None:
    r = O.run_reference(path, k, p, "k_cops_visibility_stay" + code, timeout=900)
    if r["table"] is None:
        print(f"  skip {name} k={k} p={p} stay{code}: no table file")
        return None
    cop, rob = RULES[code]
    return {"graph": name, "matrix": os.path.relpath(path, HERE), "k": k, "p": p,
            "cop_stay": cop, "robber_stay": rob, "pass_counts": r["pass_counts"],
            "base_captures": r["base_captures"], "result": r["result"], "positions": r["positions"],
            "capture_plies": r["capture_plies"],
            "sha_states": hashlib.sha256(r["table"]["states"].tobytes()).hexdigest()}


def main() -> None:
    if not O.ref_available("k_cops_visibility_stay11"):
        raise SystemExit("stay-rule reference binaries missing: run oracle/build_ref.sh first")
    out = []
    for name in SMALL:
        path = os.path.join(HERE, "matrices", name + ".txt")
        n = G.load_matrix(path).n
        for k in (1, 2, 3):
            for p in (1, 2):
                if math.comb(n + k - 1, k) * n * 2 * p > STATE_CAP:
                    continue
                for code in RULES:
                    c = case(path, name, k, p, code)
                    if c:
                        out.append(c)
        print(name, len(out), flush=True)
    for name, make, k in LARGE:
        path = os.path.join(HERE, "graphs", name + ".txt")
        if not os.path.exists(path):
            G.save_matrix(make(), path)
        for code in RULES:
            c = case(path, name, k, 1, code)
            if c:
                c["large"] = True
                out.append(c)
                print(name, code, c["pass_counts"], flush=True)
    with open(os.path.join(HERE, "stay_tables.json"), "w") as f:
        json.dump({"generated_by": "tests/golden/make_stay_tables.py", "cases": out}, f, indent=1)
    print("wrote", len(out), "cases")


if __name__ == "__main__":
    main()
