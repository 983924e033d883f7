"""Python host API over the C ABI: contexts, phase-by-phase solvers and whole solves.

The phase methods mirror the reference's solver contract (app/main.cpp:11-16):
``Solver(...)`` is buildAuxGraph, ``init()`` initializeCaptures, ``run()`` mainLoop,
``verdict()`` findFinalResult and ``write_table_file()`` outputData.
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass, field

import numpy as np

from . import native as N
from .graphs import Graph


def _check(ctx_ptr, rc: int):
    if rc != N.CR_OK:
        msg = N.lib().cr_context_last_error(ctx_ptr) if ctx_ptr else b""
        raise N.CrGpuError(rc, (msg or b"").decode(errors="replace"))


class Context:
    """One device and one stream (``stream`` = a cudaStream_t handle as int, or None)."""

    def __init__(self, device: int = 0, stream: int | None = None):
        self.ptr = ctypes.c_void_p()
        rc = N.lib().cr_context_create(device, ctypes.c_void_p(stream) if stream else None,
                                       ctypes.byref(self.ptr))
        if rc != N.CR_OK:
            raise N.CrGpuError(rc, "cr_context_create failed (no usable CUDA device?)")

    def set_profiling(self, on: bool) -> None:
        _check(self.ptr, N.lib().cr_context_set_profiling(self.ptr, int(on)))

    def set_cache_limit(self, nbytes: int) -> None:
        """Bytes of freed solver buffers this context keeps for reuse (0 = none)."""
        _check(self.ptr, N.lib().cr_context_set_cache_limit(self.ptr, int(nbytes)))

    def close(self) -> None:
        if self.ptr:
            N.lib().cr_context_destroy(self.ptr)
            self.ptr = ctypes.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class _GraphArgs:
    """Keeps the CSR arrays alive for as long as the C struct points at them."""

    def __init__(self, g: Graph):
        self.row_ptr, self.col = g.csr()
        if self.col.size == 0:
            self.col = np.zeros(1, dtype=np.uint16)
        self.struct = N.CrGraph(g.n, self.row_ptr.ctypes.data_as(N.c_u32p),
                                self.col.ctypes.data_as(N.c_u16p))


@dataclass
class Verdict:
    win: bool
    capture_plies: int
    best_config: int
    positions: tuple = field(default_factory=tuple)


def _verdict(v: N.CrVerdict, k: int) -> Verdict:
    return Verdict(bool(v.win), int(v.capture_plies), int(v.best_config),
                   tuple(int(v.positions[i]) for i in range(k)) if v.win else ())


class Solver:
    """A device state store for one (graph, k, p, rules) solve."""

    def __init__(self, ctx: Context, graph: Graph, k: int, p: int = 1, rules: int = N.CR_RULES_V1):
        self.ctx, self.graph, self.k, self.p, self.rules = ctx, graph, k, p, rules
        self._g = _GraphArgs(graph)
        self.ptr = ctypes.c_void_p()
        _check(ctx.ptr, N.lib().cr_solver_create(ctx.ptr, ctypes.byref(self._g.struct), k, p, rules,
                                                 ctypes.byref(self.ptr)))
        self.pass_counts: list[int] = []
        self.base_captures = 0

    # -- phases ----------------------------------------------------------------------
    def init(self) -> int:
        caps = ctypes.c_uint64()
        _check(self.ctx.ptr, N.lib().cr_solver_init(self.ptr, ctypes.byref(caps)))
        self.base_captures = int(caps.value)
        self.pass_counts = []
        return self.base_captures

    def step(self) -> int:
        f = ctypes.c_uint64()
        _check(self.ctx.ptr, N.lib().cr_solver_pass(self.ptr, ctypes.byref(f)))
        self.pass_counts.append(int(f.value))
        return int(f.value)

    def run(self) -> list[int]:
        cap = 1 << 14
        buf = np.zeros(cap, dtype=np.uint64)
        passes = ctypes.c_int32()
        _check(self.ctx.ptr, N.lib().cr_solver_run(self.ptr, buf.ctypes.data_as(N.c_u64p), cap,
                                                   ctypes.byref(passes)))
        self.pass_counts = [int(x) for x in buf[: passes.value]]
        return self.pass_counts

    def verdict(self) -> Verdict:
        v = N.CrVerdict()
        _check(self.ctx.ptr, N.lib().cr_solver_verdict(self.ptr, ctypes.byref(v)))
        return _verdict(v, self.k)

    # -- outputs ---------------------------------------------------------------------
    def sizes(self) -> N.CrTableSizes:
        s = N.CrTableSizes()
        _check(self.ctx.ptr, N.lib().cr_solver_sizes(self.ptr, ctypes.byref(s)))
        return s

    def stats(self) -> N.CrSolveStats:
        s = N.CrSolveStats()
        _check(self.ctx.ptr, N.lib().cr_solver_stats(self.ptr, ctypes.byref(s)))
        return s

    def v2_hash_stats(self) -> N.CrV2HashStats:
        """Cloud-table counts of a v2 solve with p >= 3 (capacity 0 otherwise)."""
        s = N.CrV2HashStats()
        _check(self.ctx.ptr, N.lib().cr_solver_v2_hash_stats(self.ptr, ctypes.byref(s)))
        return s

    def set_forms(self, mask: int) -> None:
        """Restrict a v1 solve to a subset of its kernel forms (N.CR_FORM_*); the results do
        not depend on the mask."""
        _check(self.ctx.ptr, N.lib().cr_solver_set_forms(self.ptr, mask))

    def set_v2_hash_capacity(self, slots: int) -> None:
        """Resize the v2 cloud table (0 = none); results do not depend on its size."""
        _check(self.ctx.ptr, N.lib().cr_solver_set_v2_hash_capacity(self.ptr, slots))

    def states(self, out: np.ndarray | None = None) -> np.ndarray:
        nbytes = int(self.sizes().num_states)
        if out is None:
            out = np.empty(nbytes, dtype=np.uint8)
        _check(self.ctx.ptr, N.lib().cr_solver_read_states(self.ptr, out.ctypes.data_as(N.c_u8p), out.nbytes))
        return out

    def device_states(self) -> tuple[int, int]:
        p = ctypes.c_void_p()
        n = ctypes.c_size_t()
        _check(self.ctx.ptr, N.lib().cr_solver_device_states(self.ptr, ctypes.byref(p), ctypes.byref(n)))
        return int(p.value or 0), int(n.value)

    def configs(self) -> np.ndarray:
        s = self.sizes()
        out = np.empty(int(s.config_count) * self.k, dtype=np.uint8)
        _check(self.ctx.ptr, N.lib().cr_solver_read_configs(self.ptr, out.ctypes.data_as(N.c_u8p), out.nbytes))
        return out

    def transitions(self) -> tuple[np.ndarray, np.ndarray]:
        total = ctypes.c_uint64()
        _check(self.ctx.ptr, N.lib().cr_solver_build_transitions(self.ptr, ctypes.byref(total)))
        s = self.sizes()
        heads = np.empty(int(s.config_count) + 1, dtype=np.uint64)
        data = np.empty(max(int(total.value), 1), dtype=np.uint64)
        _check(self.ctx.ptr, N.lib().cr_solver_read_transitions(
            self.ptr, heads.ctypes.data_as(N.c_u64p), heads.size, data.ctypes.data_as(N.c_u64p), data.size))
        return heads, data[: int(total.value)]

    def perfect_game(self, cap: int = 1024) -> tuple[list, bool]:
        """The perfect game of a solved p = 1 table (cr_solver_perfect_game): the positions
        (configuration id, robber vertex) after each ply, starting position first, and whether
        the walk ended in a capture.  Empty for a LOSS."""
        cfg = np.zeros(cap, dtype=np.int64)
        rob = np.zeros(cap, dtype=np.int32)
        cnt, capt = ctypes.c_int32(), ctypes.c_int32()
        _check(self.ctx.ptr, N.lib().cr_solver_perfect_game(
            self.ptr, cfg.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)),
            rob.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)), cap, ctypes.byref(cnt), ctypes.byref(capt)))
        return [(int(cfg[i]), int(rob[i])) for i in range(cnt.value)], bool(capt.value)

    def write_table_file(self, path: str) -> None:
        _check(self.ctx.ptr, N.lib().cr_solver_write_table_file(self.ptr, path.encode()))

    def load_table_file(self, path: str) -> None:
        """A table file of this solve back into the device store (a solved table)."""
        _check(self.ctx.ptr, N.lib().cr_solver_load_table_file(self.ptr, path.encode()))

    def close(self) -> None:
        if self.ptr:
            N.lib().cr_solver_destroy(self.ptr)
            self.ptr = ctypes.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


@dataclass
class Result:
    states: np.ndarray
    pass_counts: list
    base_captures: int
    verdict: Verdict
    stats: N.CrSolveStats


def solve(ctx: Context, graph: Graph, k: int, p: int = 1, rules: int = N.CR_RULES_V1,
          with_states: bool = True) -> Result:
    """Build, initialise, run to the fixed point and read the verdict (and table)."""
    with Solver(ctx, graph, k, p, rules) as s:
        caps = s.init()
        counts = s.run()
        v = s.verdict()
        st = s.states() if with_states else None
        return Result(st, counts, caps, v, s.stats())


def game_lines(configs: np.ndarray, best: int, max_plies: int, positions: list) -> list:
    """The perfect game as the reference's extractor prints it (util/perfect_game_extractor.py
    :91-165, from its 'Optimal Cop Start' line on); configs = the [C][k] configuration table."""
    show = lambda c: str(np.asarray(configs[c], dtype=np.uint8))
    out = ["", f"Optimal Cop Start: {show(best)} | Max Plys: {max_plies}", "", "--- PERFECT GAME PATH ---"]
    i = 0
    while i < len(positions):
        c, r = positions[i]
        if r in set(int(x) for x in configs[c]):
            out.append(f"Ply {i}: Game Over! Robber captured at node {r}.")
            break
        out.append(f"Ply {i} [Cop Turn]: Cops at {show(c)} | Robber at {r}")
        if i + 1 >= len(positions):
            break
        c, r = positions[i + 1]
        if r in set(int(x) for x in configs[c]):
            out.append(f"Ply {i + 1}: Cops moved to {show(c)} and CAPTURED the robber!")
            break
        out.append(f"Ply {i + 1} [Robber Turn]: Cops at {show(c)} | Robber at {r}")
        i += 2
    return out


def footprint(n: int, k: int, p: int = 1, rules: int = N.CR_RULES_V1) -> int:
    return int(N.lib().cr_solver_footprint(n, k, p, rules))


def parse_matrix(text: bytes) -> Graph:
    """Parse matrix text with the library's own parser (Graph::Graph semantics)."""
    L = N.lib()
    n = ctypes.c_int32()
    nnz = ctypes.c_size_t()
    rc = L.cr_graph_parse(text, len(text), ctypes.byref(n), None, None, 0, ctypes.byref(nnz))
    if rc:
        raise N.CrGpuError(rc, "cr_graph_parse")
    rp = np.zeros(n.value + 1, dtype=np.uint32)
    col = np.zeros(max(nnz.value, 1), dtype=np.uint16)
    rc = L.cr_graph_parse(text, len(text), ctypes.byref(n), rp.ctypes.data_as(N.c_u32p),
                          col.ctypes.data_as(N.c_u16p), col.size, ctypes.byref(nnz))
    if rc:
        raise N.CrGpuError(rc, "cr_graph_parse")
    adj = np.zeros((n.value, n.value), dtype=np.uint8)
    for v in range(n.value):
        adj[v, col[rp[v]:rp[v + 1]]] = 1
    return Graph(adj)


@dataclass
class BatchOutput:
    cop_numbers: list            # per graph: first winning k, 0 = none up to kmax
    results: list                # per graph, per k: dict of the cr_batch_result fields
    stats: N.CrBatchStats


def batch_solve(ctx: Context, graphs: list, kmax: int = 3, p: int = 1, threads: int = 0) -> BatchOutput:
    """Cop numbers of many graphs in one persistent launch (cr_batch_solve)."""
    keep = [_GraphArgs(g) for g in graphs]
    arr = (N.CrGraph * len(graphs))(*[k.struct for k in keep])
    cop = (ctypes.c_int32 * len(graphs))()
    res = (N.CrBatchResult * (len(graphs) * kmax))()
    st = N.CrBatchStats()
    _check(ctx.ptr, N.lib().cr_batch_solve(ctx.ptr, arr, len(graphs), kmax, p, threads, cop, res,
                                           ctypes.byref(st)))
    fields = [f for f, _ in N.CrBatchResult._fields_ if f != "pad"]
    out = [[{f: getattr(res[g * kmax + i], f) for f in fields} for i in range(kmax)] for g in range(len(graphs))]
    return BatchOutput([int(c) for c in cop], out, st)


def solver_digest(s: Solver) -> int:
    d = ctypes.c_uint64()
    _check(s.ctx.ptr, N.lib().cr_solver_digest(s.ptr, ctypes.byref(d)))
    return int(d.value)
