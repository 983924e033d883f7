"""Command line: solve one graph on the GPU, cop numbers of many graphs, or write a seeded
synthetic graph.

  python -m copsandrobbers_gb300.cli solve GRAPH.txt -k 3 -p 1 [--rules v1|v2] [--repeat R]
  python -m copsandrobbers_gb300.cli solve --gen regular4:256:12345 -k 3
  python -m copsandrobbers_gb300.cli gen regular4:256:12345 out.txt
  python -m copsandrobbers_gb300.cli batch --er 4096:16:128:2024 --kmax 3   (cop numbers)
  python -m copsandrobbers_gb300.cli batch a.txt b.txt ... --kmax 3
  python -m copsandrobbers_gb300.cli game GRAPH.txt -k 3      (perfect game, p = 1)

Generator specs: regular4:N:SEED, er:N:MEAN_DEGREE:SEED, delaunay:N:SEED[:MEAN_DEGREE].
"""
from __future__ import annotations

import argparse
import hashlib
import sys
import time

from . import graphs as G
from . import native as N


def graph_from_spec(spec: str) -> G.Graph:
    kind, *a = spec.split(":")
    if kind == "regular4":
        return G.regular4(int(a[0]), int(a[1]))
    if kind == "er":
        return G.erdos_renyi(int(a[0]), float(a[1]), int(a[2]))
    if kind == "delaunay":
        return G.delaunay_thinned(int(a[0]), int(a[1]), float(a[2]) if len(a) > 2 else 4.5)
    raise SystemExit(f"unknown generator spec {spec!r}")


def cmd_solve(args) -> int:
    from .solver import Context, Solver

    g = graph_from_spec(args.gen) if args.gen else G.load_matrix(args.graph)
    rules = N.CR_RULES_V2 if args.rules == "v2" else N.CR_RULES_V1
    with Context(args.device) as ctx:
        ctx.set_profiling(args.profile)
        with Solver(ctx, g, args.k, args.p, rules) as s:
            for _ in range(args.repeat):
                t0 = time.perf_counter()
                caps = s.init()
                counts = s.run()
                dt = time.perf_counter() - t0
            v = s.verdict()
            st = s.stats()
            print(f"n={g.n} k={args.k} p={args.p} rules={args.rules}: base captures {caps}, passes {counts}")
            print(f"verdict: {'WIN' if v.win else 'LOSS'} start {v.positions} capture {v.capture_plies} plies")
            print(f"init {st.init_ms:.3f} ms, main loop {st.main_ms:.3f} ms, wall {dt * 1e3:.3f} ms, "
                  f"states {s.sizes().num_states}, kernel launches {st.kernel_launches}")
            if args.digest:
                print("states sha256", hashlib.sha256(s.states().tobytes()).hexdigest())
    return 0


def er_family(spec: str) -> list:
    """COUNT:NLO:NHI:SEED -> seeded connected G(n, p) graphs, n ~ U[NLO, NHI], mean degree
    ~ U[3, 6] (the batched workload's family)."""
    import numpy as np

    count, n_lo, n_hi, seed = (int(x) for x in spec.split(":"))
    rng = np.random.default_rng(seed)
    return [G.erdos_renyi(int(rng.integers(n_lo, n_hi + 1)), float(rng.uniform(3, 6)),
                          G.sub_seed(seed, i) & 0xFFFFFFFF) for i in range(count)]


def cmd_batch(args) -> int:
    from .solver import Context, batch_solve

    graphs = [G.load_matrix(f) for f in args.graphs]
    if args.er:
        graphs += er_family(args.er)
    if not graphs:
        raise SystemExit("batch needs graph files or --er COUNT:NLO:NHI:SEED")
    with Context(args.device) as ctx:
        out = batch_solve(ctx, graphs, args.kmax, 1, args.threads)
    st = out.stats
    hist = [0] * (args.kmax + 1)
    for c in out.cop_numbers:
        hist[c] += 1
    print(f"{len(graphs)} graphs, kmax {args.kmax}: {st.ms:.3f} ms, {st.states} states, "
          f"{st.states / max(st.ms, 1e-9) / 1e6:.3f} G states/s, {st.ctas} CTAs x {st.threads} threads")
    print("cop numbers (0 = above kmax):", {i: h for i, h in enumerate(hist) if h})
    if args.list:
        for i, c in enumerate(out.cop_numbers):
            print(i, graphs[i].n, c)
    return 0


def cmd_game(args) -> int:
    from .solver import Context, Solver, game_lines

    g = graph_from_spec(args.gen) if args.gen else G.load_matrix(args.graph)
    with Context(args.device) as ctx:
        with Solver(ctx, g, args.k, 1) as s:
            s.init()
            s.run()
            v = s.verdict()
            if not v.win:
                print("RESULT: LOSS. No universal win found.")
                return 0
            walk, _ = s.perfect_game()
            cfg = s.configs().reshape(-1, args.k)
    print("\n".join(game_lines(cfg, v.best_config, v.capture_plies, walk)))
    return 0


def cmd_gen(args) -> int:
    G.save_matrix(graph_from_spec(args.spec), args.out)
    return 0


def main(argv=None) -> int:
    ap = argparse.ArgumentParser(prog="copsandrobbers_gb300.cli", description=__doc__.split("\n")[0])
    sub = ap.add_subparsers(dest="cmd", required=True)
    s = sub.add_parser("solve")
    s.add_argument("graph", nargs="?")
    s.add_argument("--gen")
    s.add_argument("-k", type=int, required=True)
    s.add_argument("-p", type=int, default=1)
    s.add_argument("--rules", choices=["v1", "v2"], default="v1")
    s.add_argument("--device", type=int, default=0)
    s.add_argument("--repeat", type=int, default=1)
    s.add_argument("--profile", action="store_true")
    s.add_argument("--digest", action="store_true")
    s.set_defaults(fn=cmd_solve)
    b = sub.add_parser("batch")
    b.add_argument("graphs", nargs="*")
    b.add_argument("--er")
    b.add_argument("--kmax", type=int, default=3)
    b.add_argument("--threads", type=int, default=0, help="threads per CTA (0 = autotune)")
    b.add_argument("--device", type=int, default=0)
    b.add_argument("--list", action="store_true")
    b.set_defaults(fn=cmd_batch)
    gm = sub.add_parser("game")
    gm.add_argument("graph", nargs="?")
    gm.add_argument("--gen")
    gm.add_argument("-k", type=int, required=True)
    gm.add_argument("--device", type=int, default=0)
    gm.set_defaults(fn=cmd_game)
    g = sub.add_parser("gen")
    g.add_argument("spec")
    g.add_argument("out")
    g.set_defaults(fn=cmd_gen)
    args = ap.parse_args(argv)
    if args.cmd in ("solve", "game") and not (args.graph or args.gen):
        ap.error(f"{args.cmd} needs GRAPH.txt or --gen SPEC")
    return args.fn(args)


if __name__ == "__main__":
    sys.exit(main())
