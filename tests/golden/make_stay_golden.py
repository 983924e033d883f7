"""Golden verdicts of the stay-allowed game: runs the reference's multithreaded legacy solver
(legacy/src/k_cops_4.cpp, built unchanged into oracle/_ref/ by oracle/build_ref.sh), whose
cops and robber may both stay, on the reference's own matrices, and stores its verdict and the
start it prints (the first configuration that wins against every robber start).

    python tests/golden/make_stay_golden.py   ->  tests/golden/stay_verdicts.json
"""
import json
import math
import os
import re
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
EXE = os.path.join(ROOT, "oracle", "_ref", "k_cops_4")
GRAPHS = ["peterson", "petersen", "grid9", "grid36", "cycle5", "cycle10", "dodecahedron", "planar8",
          "planar32", "tree7", "line10", "robertson", "rooks", "outerplanar8", "outerplanar32",
          "dismantleable19", "dismantleable48"]


def main():
    out = []
    for name in GRAPHS:
        path = os.path.join(HERE, "matrices", f"{name}.txt")
        if not os.path.exists(path):
            continue
        n = len(open(path).readline().strip())
        for k in (1, 2, 3):
            if math.comb(n + k - 1, k) * n > 3_000_000:
                continue
            res = subprocess.run([EXE, path, str(k)], capture_output=True, text=True, timeout=600).stdout
            m = re.search(r"RESULT: (WIN|LOSS)", res)
            pos = re.search(r"Optimal Cop Start Positions: \(([^)]*)\)", res)
            out.append({"graph": name, "k": k, "result": m.group(1),
                        "start": [int(x) for x in pos.group(1).split(",")] if pos else None})
            print(name, k, out[-1]["result"], out[-1]["start"])
    with open(os.path.join(HERE, "stay_verdicts.json"), "w") as f:
        json.dump(out, f, indent=1)


if __name__ == "__main__":
    sys.exit(main())
