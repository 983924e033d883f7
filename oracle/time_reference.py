"""Times the reference's own solvers (built unchanged by oracle/build_ref.sh) on bounded cases of
the large-solve workload, on the machine this runs on, and writes oracle/reference_timings.json.

The GPU host cannot run them: the reference's sources stay in the reference tree (they are not
shipped with this repository) and the binaries built here are x86-64 while that host is Arm.
bench.py reports this record next to its own CPU baseline, with the machine it came from.

  k_cops_4           legacy/src/k_cops_4.cpp, multithreaded (all hardware threads), stay-allowed
                     rules (a different game: throughput and verdict only), on the n=255 twin of
                     the large workload (4-regular, seed 12345; the reference's uint8 vertex
                     format stops at 255)
  k_cops_visibility  solvers/k_cops_visibility.cpp (the v1 solver the GPU path restates), one
                     thread, on the same generator at n=128 (the n=255 solve takes 25 minutes)

    python oracle/time_reference.py
"""
import json
import os
import platform
import re
import subprocess
import sys
import tempfile
import time

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
sys.path[0] = ROOT   # not this directory: its oracle.py would shadow the package

from copsandrobbers_gb300 import graphs as G  # noqa: E402
from oracle import oracle as O  # noqa: E402


def main():
    out = {"machine": {"cpu": platform.processor() or platform.machine(), "cores": os.cpu_count(),
                       "python_platform": platform.platform()},
           "note": "measured where the reference tree is available (not the GPU host)", "runs": []}
    n255 = os.path.join(ROOT, "tests", "golden", "graphs", "regular4_n255_s12345.txt")
    t = time.perf_counter()
    res = subprocess.run([os.path.join(HERE, "_ref", "k_cops_4"), n255, "3"], capture_output=True, text=True,
                         timeout=900).stdout
    wall = time.perf_counter() - t
    states = 2 * 255 * G.n_configs(255, 3) if hasattr(G, "n_configs") else None
    if states is None:
        from math import comb
        states = 2 * 255 * comb(257, 3)
    out["runs"].append({"solver": "k_cops_4 (legacy, stay-allowed rules)", "threads": os.cpu_count(),
                        "graph": "regular4 n=255 seed 12345", "k": 3, "states": states, "wall_s": round(wall, 2),
                        "states_per_s": states / wall,
                        "result": (re.search(r"RESULT: (WIN|LOSS)", res) or [None, None])[1]})
    with tempfile.TemporaryDirectory() as tmp:
        path = os.path.join(tmp, "regular4_n128_s12345.txt")
        G.save_matrix(G.regular4(128, 12345), path)
        t = time.perf_counter()
        r = O.run_reference(path, 3, 1, "k_cops_visibility", timeout=1800, keep_file=False)
        wall = time.perf_counter() - t
    from math import comb
    states = comb(130, 3) * 128 * 2
    out["runs"].append({"solver": "k_cops_visibility (v1)", "threads": 1, "graph": "regular4 n=128 seed 12345",
                        "k": 3, "p": 1, "states": states, "main_loop_s": r["mainloop_s"], "wall_s": round(wall, 2),
                        "states_per_s": states / r["mainloop_s"], "passes": len(r["pass_counts"]),
                        "result": r["result"]})
    with open(os.path.join(HERE, "reference_timings.json"), "w") as f:
        json.dump(out, f, indent=1)
    print(json.dumps(out, indent=1))


if __name__ == "__main__":
    main()
