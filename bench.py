#!/usr/bin/env python3
"""Benchmark of the k-cop retrograde solve on one GB300 (replicas when --gpus N > 1).

Workload (default "large"): the seeded connected 4-regular graph on n=256 vertices
(configuration model, seed 12345), k=3 cops, full visibility (p=1), v1 rules -- the large
single solve.  S = C(258,3) * 256 * 2 = 1,448,476,672 states.

A step is one whole solve with the graph resident in HBM: initializeCaptures plus mainLoop
to the fixed point (every pass, with its host read of the pass count).  The state store
(2.0 GB) is larger than L2, so no flush is needed between steps.

  value   resolved states/s = S * steps / device time, CUDA events on the solver's stream
  e2e     the same metric through the public C ABI call cr_solve() from host CSR arrays in
          pinned memory to the states table back in pinned host memory, every step
  roofline  the dominant kernel, k_init_pass1 (initializeCaptures and pass 1 in one sweep):
          algorithmic bytes per launch / its CUDA-event time; "solve" gives the whole solve's
          algorithmic state-store bytes / device time per solve
  cpu_baseline  the oracle's C restatement of the reference sweep on all host cores, timed on
          a bounded sample (one pass over a slice of the configurations), scaled to a solve

--impl reference times that same CPU restatement as the reference arm (the reference itself
cannot be built on the GPU host: its sources are not there).
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

LARGE = {"workload": "large single solve: seeded connected 4-regular graph, n=256 (configuration "
                     "model, seed 12345), k=3 cops, p=1, v1 rules",
         "n": 256, "k": 3, "p": 1, "rules": "v1", "graph_seed": 12345,
         "l2": "state store 2.0 GB > L2 (129 MB): no flush needed"}
METRIC = "resolved states/s"


def max_over_ranks(ms: float, world: int, device: str = "cuda") -> float:
    """The slowest rank's time (every rank gets it): the job's time for N replicas."""
    if world <= 1:
        return ms
    import torch
    import torch.distributed as dist

    t = torch.tensor([ms], device=device, dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replicas_value(states_per_step: int, steps: int, world: int, max_ms: float) -> float:
    """Whole-job throughput of N replicas: the states all ranks solved over the slowest rank's time."""
    return states_per_step * steps * world / (max_ms / 1e3)


def dist_info():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.lines: list[str] = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.device}", f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self) -> dict:
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [x.strip() for x in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx.append(float(parts[2]))
            except ValueError:
                continue
            for nm, val in zip(names, parts[5:9]):
                if val.lower() in ("active", "1"):
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def measured_peak_hbm() -> tuple[float, str]:
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


def solve_dram_bytes() -> float | None:
    """Measured DRAM bytes of one solve step (ncu over every launch) from the committed summary."""
    path = os.path.join(ROOT, "profiles", "large_solve_n256_launches.md")
    try:
        for line in open(path):
            if line.startswith("solve_dram_bytes:"):
                return float(line.split(":")[1])
    except OSError:
        pass
    return None


def traffic_per_launch() -> float | None:
    """DRAM bytes per k_init_pass1 launch from the committed ncu summary, if present."""
    path = os.path.join(ROOT, "profiles", "k_init_pass1_large_n256.md")
    try:
        for line in open(path):
            if line.startswith("traffic_bytes_per_launch:"):
                return float(line.split(":")[1])
    except OSError:
        pass
    return None


def reference_code_timings() -> dict | None:
    """The reference's own solvers timed by oracle/time_reference.py where the reference tree is
    (its sources do not ship with this repository, and its x86-64 builds do not run on the Arm
    GPU host): a record with the machine it came from, not a measurement of this run."""
    path = os.path.join(ROOT, "oracle", "reference_timings.json")
    try:
        with open(path) as f:
            return json.load(f)
    except (OSError, ValueError):
        return None


def cpu_baseline(graph, k: int, p: int, passes: int, budget_s: float = 20.0) -> dict:
    """The oracle's restatement of the reference sweep on all host cores over a bounded sample."""
    from oracle import oracle as O

    samp = O.SweepSample(graph, k, p)
    cores = os.cpu_count() or 1
    C = samp.count
    slice_cfg = max(1, C // 64)
    done_cfg, t_total, c0 = 0, 0.0, 0
    while t_total < budget_s and c0 < C:
        c1 = min(C, c0 + slice_cfg)
        t = time.perf_counter()
        samp.run(c0, c1, cores)
        t_total += time.perf_counter() - t
        done_cfg += c1 - c0
        c0 = c1
    swept = done_cfg * graph.n * 2 * p
    rate = swept / t_total / passes
    return {"value": rate, "unit": METRIC, "cores": cores, "kind": "port",
            "sample": f"one v1 pass (all {2 * p} columns) over {done_cfg} of {C} configurations "
                      f"({swept} states, {t_total:.1f} s), scaled by the solve's {passes} passes",
            "reference_code": reference_code_timings()}


def batched_workload(ctx, count: int = 4096) -> dict:
    """Cop numbers of `count` seeded connected G(n, p) graphs, n ~ U[16, 128], mean degree
    ~ U[3, 6], k = 1, 2, 3 in order: one persistent launch (cr_batch_solve) against the plain
    form -- one solve per (graph, k) through the public API on the same context, whose block
    cache reuses the state store from solve to solve -- over every (graph, k) the batch solved.
    The plain form's timed loop keeps each solve's pass counts; every table digest is taken in
    a second, untimed loop and compared with the batch's, as is every pass-count hash."""
    import numpy as np

    from copsandrobbers_gb300 import graphs as G
    from copsandrobbers_gb300 import native as N
    from copsandrobbers_gb300.solver import Solver, batch_solve, solver_digest

    rng = np.random.default_rng(2024)
    graphs = [G.erdos_renyi(int(rng.integers(16, 129)), float(rng.uniform(3, 6)),
                            G.sub_seed(2024, i) & 0xFFFFFFFF) for i in range(count)]
    batch_solve(ctx, graphs, 3, 1, 0)  # warm-up (the autotuner calibrates on this batch)
    out = batch_solve(ctx, graphs, 3, 1, 0)
    batched = out.stats.states / (out.stats.ms / 1e3)
    jobs = [(gi, k) for gi in range(count) for k in range(1, 4) if out.results[gi][k - 1]["solved"]]
    for gi, k in jobs[:32]:   # warm-up of the plain form (fills the context's block cache)
        with Solver(ctx, graphs[gi], k, 1) as s:
            s.init()
            s.run()
    hashes = []
    t0 = time.perf_counter()
    for gi, k in jobs:
        with Solver(ctx, graphs[gi], k, 1) as s:
            s.init()
            hashes.append(N.pass_hash(s.run()))
    plain_s = time.perf_counter() - t0
    states = sum(int(out.results[gi][k - 1]["states"]) for gi, k in jobs)
    mismatch = 0
    for (gi, k), ph in zip(jobs, hashes):
        r = out.results[gi][k - 1]
        with Solver(ctx, graphs[gi], k, 1) as s:
            s.init()
            s.run()
            dg = solver_digest(s)
        mismatch += int(dg != r["digest"] or ph != r["pass_hash"])
    plain = states / plain_s
    return {"workload": f"{count} connected G(n,p), n~U[16,128], mean degree~U[3,6], k=1..3 until WIN",
            "batched_states_per_s": batched, "plain_states_per_s": plain,
            "batched_over_plain": batched / plain, "batched_ms": out.stats.ms, "plain_ms": plain_s * 1e3,
            "states": int(out.stats.states), "ctas": int(out.stats.ctas), "threads": int(out.stats.threads),
            "busy_frac": float(out.stats.busy_frac), "tail_ms": float(out.stats.tail_ms),
            "plain_sample_graphs": count, "plain_solves": len(jobs), "table_mismatches": mismatch,
            "plain_form": "one Solver per (graph, k): create, initializeCaptures, mainLoop, destroy; "
                          "store blocks reused through the context's cache; digests outside the timed loop",
            "cop_number_histogram": [int(x) for x in np.bincount(out.cop_numbers, minlength=4)]}


def limited_visibility_workload(ctx) -> dict:
    """v2 rules on the seeded Delaunay-thinned graph, n=199, mean degree 4.5, k=2, p=3."""
    from copsandrobbers_gb300 import graphs as G
    from copsandrobbers_gb300 import native as N
    from copsandrobbers_gb300.solver import Solver

    g = G.delaunay_thinned(199, 2024)
    with Solver(ctx, g, 2, 3, N.CR_RULES_V2) as s:
        s.init()
        s.run()
        s.init()
        t0 = time.perf_counter()
        counts = s.run()
        dt = time.perf_counter() - t0
        v = s.verdict()
        st = s.stats()
        S = int(s.sizes().num_states)
    return {"workload": "Delaunay-thinned n=199 (seed 2024, mean degree 4.5), k=2, p=3, v2 rules",
            "states": S, "solve_s": dt, "states_per_s": S / dt, "passes": len(counts),
            "device_ms": st.main_ms, "verdict": "WIN" if v.win else "LOSS",
            "reference": "the reference v2 solver did not finish this graph at p=2 within 600 s"}


def serving_workload(count: int, rate: float, workers: int = 16) -> dict:
    """A seeded Poisson stream of solve requests through the solve server (cr_server_*):
    4-regular / G(n, 4/(n-1)) / Delaunay-thinned graphs, n log-uniform in [20, 400], k in
    {1, 2, 3}, 10% with visibility period p in [2, 4] (half of those under the v2 rules with
    k <= 2, p <= 3, n <= 200);
    admission by device footprint, tables resident until the client releases them."""
    from copsandrobbers_gb300.serving import Server, request_stream, run_stream

    t0 = time.perf_counter()
    reqs = request_stream(count, rate_per_s=rate, seed=12)
    gen_s = time.perf_counter() - t0
    with Server(0, 0, workers=workers) as srv:
        run_stream(srv, request_stream(40, rate_per_s=1e6, seed=99))   # warm-up
        out = run_stream(srv, reqs)
    failed = sum(1 for r in out["results"] if r["status"] != 0)
    lat_q = sorted(float(r["queue_ms"]) for r in out["results"])
    return {"workload": f"{count} Poisson arrivals at {rate:g} requests/s (seed 12): 4-regular / "
                        "G(n,p) mean degree 4 / Delaunay-thinned, n log-uniform in [20,400], k in {1,2,3}, "
                        "10% with p in [2,4] (half of them v2 rules with k <= 2, p <= 3, n <= 200)",
            "rate_per_s": rate, "requests": count, "workers": workers, "wall_s": out["wall_s"],
            "p50_ms": out["p50_ms"], "p99_ms": out["p99_ms"], "mean_ms": out["mean_ms"],
            "queue_p50_ms": lat_q[len(lat_q) // 2] if lat_q else None,
            "states": out["states"], "states_per_s": out["states_per_s"], "failed": failed,
            "max_running": out["stats"]["max_running"],
            "peak_memory_in_use": out["stats"]["peak_memory_in_use"], "generate_s": gen_s}


def run_reference(args) -> None:
    rank, world, _ = dist_info()
    if rank != 0:
        return
    from copsandrobbers_gb300 import graphs as G
    from oracle import oracle as O

    g = G.regular4(LARGE["n"], LARGE["graph_seed"])
    k, p = LARGE["k"], LARGE["p"]
    samp = O.SweepSample(g, k, p)
    cores = os.cpu_count() or 1
    C = samp.count
    slice_cfg = max(1, C // 64)
    # the solve's pass count, from the oracle's full solve of this graph (tests/golden/large.json;
    # the GPU arm finds the same): one pass over a slice of the configurations is timed per step
    with open(os.path.join(ROOT, "tests", "golden", "large.json")) as f:
        passes = len(json.load(f)["n256"]["pass_counts"])

    def step(i):
        c0 = (i * slice_cfg) % C
        c1 = min(C, c0 + slice_cfg)
        t = time.perf_counter()
        samp.run(c0, c1, cores)
        return time.perf_counter() - t, (c1 - c0) * g.n * 2 * p

    for i in range(args.warmup):
        step(i)
    t_sum, s_sum = 0.0, 0
    for i in range(args.steps):
        dt, st = step(args.warmup + i)
        t_sum += dt
        s_sum += st
    value = s_sum / t_sum / passes
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "states/s",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1e3 * t_sum / max(args.steps, 1), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "u8", "data": "synthetic (seeded generator)", "config": LARGE,
        "cpu_baseline": {"value": value, "unit": "states/s", "cores": cores, "kind": "port",
                         "sample": f"per step one v1 pass over {slice_cfg} of {C} configurations, "
                                   f"scaled by the solve's {passes} passes",
                         "reference_code": reference_code_timings()},
        "e2e": {"value": value, "unit": "states/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def run_gpu(args) -> None:
    import torch

    rank, world, local = dist_info()
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    torch.cuda.set_device(local)
    from copsandrobbers_gb300 import graphs as G
    from copsandrobbers_gb300 import native as N
    from copsandrobbers_gb300.solver import Context, Solver

    g = G.regular4(LARGE["n"], LARGE["graph_seed"])
    k, p = LARGE["k"], LARGE["p"]
    stream = torch.cuda.Stream()
    ctx = Context(local, stream.cuda_stream)
    solver = Solver(ctx, g, k, p, N.CR_RULES_V1)
    sizes = solver.sizes()
    S = int(sizes.num_states)

    def barrier():
        if world > 1:
            torch.distributed.barrier()

    # warm-up solves
    for _ in range(args.warmup):
        solver.init()
        solver.run()
    launches_per_step = int(solver.stats().kernel_launches)
    passes = len(solver.pass_counts)

    # timed region: K whole solves on the solver's stream
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    barrier()
    k_launch_ms = []   # k_init_pass1's own CUDA-event time in each timed solve
    with ClockSampler(local) as clocks:
        ev0.record(stream)
        for _ in range(args.steps):
            solver.init()
            solver.run()
            k_launch_ms.append(float(solver.stats().init_ms))
        ev1.record(stream)
        torch.cuda.synchronize()
    barrier()
    ms = max_over_ranks(ev0.elapsed_time(ev1), world)
    value = replicas_value(S, args.steps, world, ms)
    verdict = solver.verdict()

    # roofline of the dominant kernel, k_init_pass1 (initializeCaptures and pass 1 in one
    # sweep): its launch time comes from CUDA events around it on the solver's stream
    # (stats.init_ms), averaged over the K timed solves
    st = solver.stats()
    C, n = int(sizes.config_count), int(sizes.n)
    rw = (n + 31) // 32
    rwp = rw if rw <= 2 else (rw + 3) // 4 * 4
    slots = int(st.slots)
    k_ms = statistics.mean(k_launch_ms)
    # algorithmic bytes of one k_init_pass1 launch: every table byte written once (S), both
    # marked bit planes written (2 * C * rwp * 4) and both flag planes (2 * C); the column-1
    # frontier rows of the few configurations that changed are left out (a lower bound)
    k_bytes = S + 2 * C * rwp * 4 + 2 * C
    achieved = k_bytes / (k_ms / 1e3) / 1e9 if k_ms > 0 else None
    peak, peak_kind = measured_peak_hbm()
    traffic = traffic_per_launch()
    # whole-solve algorithmic bytes (the state store's minimal traffic): per level both
    # resolved bit planes read (S/8), the frontier plane read and the next written (S/16 each),
    # the resolved bits written (S/8) = 3S/8; 2 B of capture depth per resolved state; 1 B of
    # escape counter per state written and read once (S)
    resolved = 2 * int(solver.base_captures) + sum(solver.pass_counts)
    solve_bytes = passes * 3 * S / 8 + 2 * resolved + S
    solve_achieved = solve_bytes / (ms / args.steps / 1e3) / 1e9
    # the whole step, twice: by DRAM bytes measured with ncu over every launch of one solve
    # (profiles/large_solve_n256_launches.md), and by the byte model above, labelled as such
    dram = solve_dram_bytes()
    step_s = ms / args.steps / 1e3
    solve_roofline = {"dram_bytes": dram, "dram_gbs": dram / step_s / 1e9 if dram else None,
                      "dram_frac": dram / step_s / 1e9 / measured_peak_hbm()[0] if dram else None,
                      "dram_source": "ncu dram__bytes_read.sum + dram__bytes_write.sum over one solve's launches",
                      "model_bytes": solve_bytes, "model_gbs": solve_achieved,
                      "model_frac": solve_achieved / measured_peak_hbm()[0],
                      "model": "per level 3S/8 of bit planes + 2 B depth per resolved state + 1 B counter per "
                               "state (a store layout with counter arrays; not traffic of this solver)",
                      "levels": passes, "resolved_states": resolved}
    solver.close()

    # e2e: the public one-call API from pinned host CSR to the pinned host table
    import ctypes
    import numpy as np
    row_ptr, col = g.csr()
    rp_pin = torch.from_numpy(row_ptr.view(np.int32)).pin_memory()
    col_pin = torch.from_numpy(col.view(np.int16)).pin_memory()
    out_pin = torch.empty(S, dtype=torch.uint8, pin_memory=True)
    cg = N.CrGraph(n, ctypes.cast(rp_pin.data_ptr(), N.c_u32p), ctypes.cast(col_pin.data_ptr(), N.c_u16p))
    counts = np.zeros(1024, dtype=np.uint64)
    npass = ctypes.c_int32()
    vv = N.CrVerdict()
    L = N.lib()

    def e2e_step():
        rc = L.cr_solve(ctx.ptr, ctypes.byref(cg), k, p, N.CR_RULES_V1,
                        ctypes.cast(out_pin.data_ptr(), N.c_u8p), S, counts.ctypes.data_as(N.c_u64p),
                        1024, ctypes.byref(npass), ctypes.byref(vv), None)
        if rc:
            raise RuntimeError(f"cr_solve failed: {rc} {L.cr_context_last_error(ctx.ptr)}")

    for _ in range(max(1, args.warmup)):
        e2e_step()
    torch.cuda.synchronize()
    barrier()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.steps):
        e2e_step()
    e1.record(stream)
    torch.cuda.synchronize()
    barrier()
    e2e_ms = max_over_ranks(e0.elapsed_time(e1), world)
    e2e_value = replicas_value(S, args.steps, world, e2e_ms)

    line = None
    extra = {}
    if rank == 0 and not args.headline_only:
        # the other workloads of the benchmark; a failure in one is reported in its key and
        # does not take the headline line with it
        for key, run in (("batched", lambda: batched_workload(ctx)),
                         ("limited_visibility", lambda: limited_visibility_workload(ctx)),
                         ("serving", lambda: serving_workload(args.serving_requests, args.serving_rate))):
            try:
                extra[key] = run()
            except Exception as e:  # noqa: BLE001 - reported, not swallowed
                extra[key] = {"error": f"{type(e).__name__}: {e}"}
                print(f"bench: {key} workload failed: {e}", file=sys.stderr, flush=True)
    if rank == 0:
        base = cpu_baseline(g, k, p, passes) if not args.no_cpu_baseline else None
        line = {
            "metric": METRIC, "value": value, "unit": "states/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "u8",
            "data": "synthetic (seeded generator, committed as tests/golden/graphs/regular4_n256_s12345.txt)",
            "config": dict(LARGE, parallelism=f"replicas x{world}" if world > 1 else "single GPU",
                           passes=passes, verdict="WIN" if verdict.win else "LOSS"),
            "e2e": {"value": e2e_value, "unit": "states/s",
                    "h2d_bytes_per_step": int(row_ptr.nbytes + col.nbytes),
                    "d2h_bytes_per_step": int(S + 8 * len(counts) + ctypes.sizeof(vv))},
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak if achieved else None, "traffic": traffic,
                         "kernel": "k_init_pass1 (initializeCaptures + pass 1, one launch per solve)",
                         "peak_source": peak_kind, "mean_launch_ms": k_ms, "alg_bytes_per_launch": k_bytes,
                         "solve": solve_roofline},
            "cpu_baseline": base,
            "clocks": clocks.summary(),
            "gpu_launches": launches_per_step * args.steps,
        }
        line.update(extra)
        print(json.dumps(line), flush=True)
    ctx.close()
    if world > 1:
        torch.distributed.destroy_process_group()


def main() -> None:
    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["gpu", "reference"], default="gpu")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--headline-only", action="store_true",
                    help="skip the batched, limited-visibility and serving workloads")
    ap.add_argument("--serving-requests", type=int, default=20000)
    ap.add_argument("--serving-rate", type=float, default=45.0, help="requests per second")
    args = ap.parse_args()
    if args.impl == "reference":
        run_reference(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
