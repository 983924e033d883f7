"""Generate the golden fixtures from the reference solvers themselves.

Runs the reference binaries compiled by oracle/build_ref.sh (from the reference's own
sources, unchanged) on the reference's own adjacency matrices and on the seeded synthetic
graphs, and records for each (graph, k, p, solver) case what the reference printed and
wrote: pass counts, base captures, verdict, start positions, capture time, and SHA-256
digests of every section of the table file it saved.

The matrices used are copied into tests/golden/matrices/ so the fixtures travel without the
reference tree.  Re-run with:  python tests/golden/make_golden.py  (needs the reference tree, at
CR_REFERENCE_ROOT or /root/reference).
"""
from __future__ import annotations

import hashlib
import json
import os
import shutil
import sys
import time

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import oracle as O  # noqa: E402
from copsandrobbers_gb300 import graphs as G  # noqa: E402

REF_ROOT = os.environ.get("CR_REFERENCE_ROOT", "/root/reference")
REF_MATRICES = os.path.join(REF_ROOT, "assets", "matrices")
OUT_MATRICES = os.path.join(HERE, "matrices")
CASES = os.path.join(HERE, "cases.json")

SMALL = ["cycle3", "cycle5", "cycle10", "line3", "line5", "line10", "tree3", "tree7", "test",
         "grid9", "rooks", "planar8", "outerplanar8", "peterson", "robertson", "dodecahedron",
         "dismantleable19", "outerplanar32", "planar32", "grid36", "dismantleable48"]
V1_STATE_CAP = 6_000_000      # C * n * 2p states per v1 case
V2_STATE_CAP = 400_000        # C * n states per v2 case (its search is exponential in p)


def sha(b: bytes) -> str:
    return hashlib.sha256(b).hexdigest()


def n_configs(n: int, k: int) -> int:
    from math import comb
    return comb(n + k - 1, k)


def record(path: str, name: str, k: int, p: int, solver: str, timeout: float) -> dict | None:
    t0 = time.time()
    try:
        r = O.run_reference(path, k, p, solver, timeout=timeout)
    except Exception as e:  # timeout: the case is left out
        print(f"  skip {name} k={k} p={p} {solver}: {type(e).__name__}")
        return None
    tab = r["table"]
    if tab is None:
        print(f"  skip {name} k={k} p={p} {solver}: no table file")
        return None
    case = {
        "graph": name, "k": k, "p": p, "solver": solver,
        "n": int(tab["n"]), "columns": int(tab["columns"]), "config_count": int(tab["config_count"]),
        "pass_counts": r["pass_counts"], "base_captures": r["base_captures"],
        "result": r["result"], "positions": r["positions"], "capture_plies": r["capture_plies"],
        "table_file": r["table_file"],
        "sha_file": sha(tab["raw"]), "sha_states": sha(tab["states"].tobytes()),
        "sha_configs": sha(tab["configs"].tobytes()), "sha_heads": sha(tab["heads"].tobytes()),
        "sha_transitions": sha(tab["transitions"].tobytes()),
        "n_transitions": int(tab["transitions"].size),
        "ref_seconds": round(time.time() - t0, 3), "ref_mainloop_s": r["mainloop_s"],
    }
    return case


def large() -> None:
    """The large single solve's digests (minutes of CPU time; run with --large):
    n=255 by the reference binary itself (its format stops at 255 vertices), and the n=256
    product configuration by the oracle's C restatement, pinned by the n=255 agreement."""

    out = {}
    src = os.path.join(HERE, "graphs", "regular4_n255_s12345.txt")
    c = record(src, "regular4_n255_s12345", 3, 1, "k_cops_visibility", 7200)
    c["matrix"] = os.path.relpath(src, HERE)
    c["pinned_by"] = "reference binary"
    out["n255"] = c
    g = G.load_matrix(os.path.join(HERE, "graphs", "regular4_n256_s12345.txt"))
    t0 = time.time()
    sol = O.solve_v1(g, 3, 1)
    out["n256"] = {
        "graph": "regular4_n256_s12345", "matrix": "graphs/regular4_n256_s12345.txt", "k": 3, "p": 1,
        "solver": "k_cops_visibility", "n": 256, "columns": 2, "config_count": int(sol.configs.shape[0]),
        "pass_counts": sol.pass_counts, "base_captures": sol.base_captures,
        "result": "WIN" if sol.win else "LOSS", "sha_states": sha(sol.states.tobytes()),
        "sha_heads": sha(sol.heads.tobytes()), "sha_transitions": sha(sol.transitions.tobytes()),
        "n_transitions": int(sol.transitions.size), "pinned_by": "oracle (C restatement)",
        "oracle_seconds": round(time.time() - t0, 1),
    }
    with open(os.path.join(HERE, "large.json"), "w") as f:
        json.dump(out, f, indent=1)
    print("wrote large.json")


def main() -> None:
    os.makedirs(OUT_MATRICES, exist_ok=True)
    if not O.ref_available():
        raise SystemExit("reference binaries missing: run oracle/build_ref.sh first")
    cases = []
    for name in SMALL:
        src = os.path.join(REF_MATRICES, name + ".txt")
        dst = os.path.join(OUT_MATRICES, name + ".txt")
        shutil.copyfile(src, dst)
        n = G.load_matrix(dst).n
        for k in (1, 2, 3):
            for p in (1, 2, 3):
                if n_configs(n, k) * n * 2 * p <= V1_STATE_CAP:
                    c = record(dst, name, k, p, "k_cops_visibility", 120)
                    if c:
                        cases.append(c)
                if k <= 2 and n_configs(n, k) * n <= V2_STATE_CAP:
                    c = record(dst, name, k, p, "k_cops_visibility_v2", 60)
                    if c:
                        cases.append(c)
        print(f"{name}: {len(cases)} cases so far", flush=True)
    # the reference's largest in-tree board, and the seeded synthetic graphs
    extra = [("scotlandyard-all", os.path.join(REF_MATRICES, "scotlandyard-all.txt"), 2, 1, "k_cops_visibility"),
             ("delaunay_n199_s2024", os.path.join(HERE, "graphs", "delaunay_n199_s2024.txt"), 1, 1, "k_cops_visibility"),
             ("delaunay_n199_s2024", os.path.join(HERE, "graphs", "delaunay_n199_s2024.txt"), 1, 2, "k_cops_visibility_v2"),
             ("delaunay_n199_s2024", os.path.join(HERE, "graphs", "delaunay_n199_s2024.txt"), 2, 1, "k_cops_visibility_v2")]
    for name, src, k, p, solver in extra:
        if src.startswith(REF_MATRICES):
            dst = os.path.join(OUT_MATRICES, name + ".txt")
            shutil.copyfile(src, dst)
        else:
            dst = src
        c = record(dst, name, k, p, solver, 900)
        if c:
            c["matrix"] = os.path.relpath(dst, HERE)
            cases.append(c)
            print(f"{name} k={k} p={p} {solver}: {c['ref_seconds']} s", flush=True)
    for c in cases:
        c.setdefault("matrix", os.path.join("matrices", c["graph"] + ".txt"))
    with open(CASES, "w") as f:
        json.dump({"generator": "tests/golden/make_golden.py", "cases": cases}, f, indent=1)
    print(f"wrote {len(cases)} cases to {CASES}")


if __name__ == "__main__":
    if "--large" in sys.argv:
        large()
    else:
        main()
