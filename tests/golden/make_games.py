"""Golden perfect games: runs the reference's own util/perfect_game_extractor.py (imported from
the reference tree) on tables of the oracle, written in the extractor's file layout (80-byte
header of ten u64: k, N, configCount, numStates, stride, five section offsets; configs u8,
heads u64, transitions u64, states u8, then an N x (maxDegree + 1) u8 edge table terminated by
255), and stores the printed game from its 'Optimal Cop Start' line on.

    python tests/golden/make_games.py /path/to/reference   ->  tests/golden/games.json
"""
import contextlib
import importlib.util
import io
import json
import os
import struct
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
from copsandrobbers_gb300 import graphs as G  # noqa: E402
from oracle import oracle as O  # noqa: E402

CASES = [("peterson", 3), ("dodecahedron", 3), ("grid9", 2), ("planar8", 2), ("cycle5", 2),
         ("cycle10", 2), ("dismantleable48", 1), ("grid36", 2)]


def extractor_file(sol, graph, path):
    n, k, C = sol.n, sol.k, sol.configs.shape[0]
    rp, col = graph.csr()
    maxdeg = int(max(rp[1:] - rp[:-1])) if n else 0
    edges = np.full((n, maxdeg + 1), 255, dtype=np.uint8)
    for v in range(n):
        nb = col[rp[v]:rp[v + 1]]
        edges[v, :len(nb)] = nb
    cfg = sol.configs.astype(np.uint8).tobytes()
    heads = sol.heads.astype(np.uint64).tobytes()
    trans = sol.transitions.astype(np.uint64).tobytes()
    states = sol.states.tobytes()
    o1 = 80
    o2 = o1 + len(cfg)
    o3 = o2 + len(heads)
    o4 = o3 + len(trans)
    o5 = o4 + len(states)
    with open(path, "wb") as f:
        f.write(struct.pack("10Q", k, n, C, len(states), 1, o1, o2, o3, o4, o5))
        f.write(cfg + heads + trans + states + edges.tobytes())


def main():
    ref = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("CR_REFERENCE_ROOT", "/root/reference")
    spec = importlib.util.spec_from_file_location("pge", os.path.join(ref, "util", "perfect_game_extractor.py"))
    pge = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(pge)
    out = []
    with tempfile.TemporaryDirectory() as tmp:
        for name, k in CASES:
            mpath = os.path.join(HERE, "matrices", f"{name}.txt")
            g = G.load_matrix(mpath)
            sol = O.solve_v1(g, k, 1)
            path = os.path.join(tmp, "t.bin")
            extractor_file(sol, g, path)
            buf = io.StringIO()
            with contextlib.redirect_stdout(buf):
                pge.extract_perfect_game(path)
            lines = buf.getvalue().split("\n")
            if "RESULT: LOSS. No universal win found." in lines:
                game = None
            else:
                start = lines.index(next(l for l in lines if l.startswith("Optimal Cop Start"))) - 1
                game = [l for l in lines[start:]]
                while game and game[-1] == "":
                    game.pop()
            out.append({"graph": name, "k": k, "win": sol.win, "lines": game})
            print(name, k, "WIN" if sol.win else "LOSS", len(game or []), "lines")
    with open(os.path.join(HERE, "games.json"), "w") as f:
        json.dump(out, f, indent=1)


if __name__ == "__main__":
    main()
