"""Python front end of the oracle (TEST INFRASTRUCTURE ONLY).

Wraps ``libcroracle.so`` (the C restatement in ``cr_oracle.c``) and the reference binaries
compiled into ``_ref/`` by ``build_ref.sh``.  Only the tests, ``__graft_entry__.smoke()`` and
the CPU-baseline leg of ``bench.py`` import this module, and only as the oracle the GPU
results are compared with.
"""
from __future__ import annotations

import ctypes
import os
import re
import shutil
import struct
import subprocess
import tempfile
from dataclasses import dataclass, field

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
# Idle OpenMP workers sleep instead of spinning: the oracle often shares the host with other
# work (a GPU process, a reference run), where spinning barriers slow every column sweep.
os.environ.setdefault("OMP_WAIT_POLICY", "PASSIVE")
REF_DIR = os.path.join(HERE, "_ref")
_LIB = None

u64p = ctypes.POINTER(ctypes.c_uint64)
u32p = ctypes.POINTER(ctypes.c_uint32)
u16p = ctypes.POINTER(ctypes.c_uint16)
u8p = ctypes.POINTER(ctypes.c_uint8)


def build() -> None:
    subprocess.run(["make", "-s", "-C", HERE, "libcroracle.so"], check=True)


def lib():
    global _LIB
    if _LIB is None:
        path = os.path.join(HERE, "libcroracle.so")
        if not os.path.exists(path):
            build()
        L = ctypes.CDLL(path)
        L.or_config_count.restype = ctypes.c_uint64
        L.or_config_count.argtypes = [ctypes.c_int, ctypes.c_int]
        L.or_configs.argtypes = [ctypes.c_int, ctypes.c_int, u16p]
        L.or_transitions.argtypes = [ctypes.c_int, u32p, u16p, ctypes.c_int, ctypes.c_int, u16p,
                                     ctypes.c_uint64, u64p, u64p]
        L.or_v1_solve.restype = ctypes.c_int
        L.or_v1_solve.argtypes = [ctypes.c_int, u32p, u16p, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                  ctypes.c_int, u16p, ctypes.c_uint64, u64p, u64p, u8p, u64p, u64p,
                                  ctypes.c_int, ctypes.c_int]
        L.or_v2_solve.restype = ctypes.c_int
        L.or_v2_solve.argtypes = [ctypes.c_int, u32p, u16p, ctypes.c_int, ctypes.c_int, u16p,
                                  ctypes.c_uint64, u64p, u64p, u8p, u64p, u64p, ctypes.c_int,
                                  ctypes.c_int]
        L.or_v1_init.restype = ctypes.c_uint64
        L.or_v1_init.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, u16p, ctypes.c_uint64, u8p]
        L.or_v1_sweep_slice.restype = ctypes.c_uint64
        L.or_v1_sweep_slice.argtypes = [ctypes.c_int, u32p, u16p, ctypes.c_int, ctypes.c_int, u64p, u64p,
                                        u8p, ctypes.c_int64, ctypes.c_int64, ctypes.c_int]
        L.or_verdict.restype = ctypes.c_int64
        L.or_verdict.argtypes = [ctypes.c_int, ctypes.c_uint64, ctypes.c_int, u8p,
                                 ctypes.POINTER(ctypes.c_int)]
        _LIB = L
    return _LIB


def _p(a, t):
    return a.ctypes.data_as(t)


@dataclass
class Solution:
    """What one solve produces: the sections of the reference's table file and its stdout."""

    n: int
    k: int
    p: int
    columns: int
    configs: np.ndarray          # uint16 [C, k]
    heads: np.ndarray            # uint64 [C + 1]
    transitions: np.ndarray      # uint64 [heads[-1]] = next config id * n
    states: np.ndarray           # uint8 [C * n * columns]
    base_captures: int
    pass_counts: list = field(default_factory=list)
    best_config: int = -1
    capture_plies: int = 127

    @property
    def win(self) -> bool:
        return self.best_config >= 0

    def start_positions(self) -> tuple:
        return tuple(int(x) for x in self.configs[self.best_config]) if self.win else ()


def configs(n: int, k: int) -> np.ndarray:
    L = lib()
    c = L.or_config_count(n, k)
    out = np.zeros(c * k, dtype=np.uint16)
    L.or_configs(n, k, _p(out, u16p))
    return out.reshape(c, k)


def transitions(graph, k: int, cfg: np.ndarray, cop_stay: bool = False):
    L = lib()
    row_ptr, col = graph.csr()
    col = np.ascontiguousarray(col if col.size else np.zeros(1, np.uint16))
    c = cfg.shape[0]
    heads = np.zeros(c + 1, dtype=np.uint64)
    L.or_transitions(graph.n, _p(row_ptr, u32p), _p(col, u16p), k, int(cop_stay),
                     _p(np.ascontiguousarray(cfg), u16p), c, _p(heads, u64p), None)
    data = np.zeros(max(int(heads[-1]), 1), dtype=np.uint64)
    L.or_transitions(graph.n, _p(row_ptr, u32p), _p(col, u16p), k, int(cop_stay),
                     _p(np.ascontiguousarray(cfg), u16p), c, _p(heads, u64p), _p(data, u64p))
    return heads, data[: int(heads[-1])]


def solve_v1(graph, k: int, p: int = 1, threads: int = 0, max_passes: int = 4096,
             cop_stay: bool = False, robber_stay: bool = False) -> Solution:
    """v1 (solvers/k_cops_visibility.cpp) restated: the 2p-column sweep to its fixed point.
    cop_stay / robber_stay: the self-edge rules of AuxGraph.h:203-205 and
    k_cops_visibility.cpp:253-255 (off in the reference's solvers)."""
    L = lib()
    cfg = configs(graph.n, k)
    heads, trans = transitions(graph, k, cfg, cop_stay)
    cols = 2 * p
    states = np.empty(cfg.shape[0] * graph.n * cols, dtype=np.uint8)
    row_ptr, col = graph.csr()
    col = np.ascontiguousarray(col if col.size else np.zeros(1, np.uint16))
    caps = ctypes.c_uint64(0)
    counts = np.zeros(max_passes, dtype=np.uint64)
    tr = trans if trans.size else np.zeros(1, np.uint64)
    passes = L.or_v1_solve(graph.n, _p(row_ptr, u32p), _p(col, u16p), k, p, int(cop_stay), int(robber_stay),
                           _p(cfg, u16p), cfg.shape[0], _p(heads, u64p), _p(tr, u64p),
                           _p(states, u8p), ctypes.byref(caps), _p(counts, u64p), max_passes,
                           threads)
    if passes < 0:
        raise RuntimeError(f"oracle v1 failed ({passes})")
    sol = Solution(graph.n, k, p, cols, cfg, heads, trans, states, int(caps.value),
                   [int(x) for x in counts[:passes]])
    _verdict(sol)
    return sol


def solve_v2(graph, k: int, p: int, threads: int = 0, max_passes: int = 4096) -> Solution:
    """v2 (solvers/k_cops_visibility_v2.cpp) restated: snapshot passes of the macro-turn search."""
    L = lib()
    cfg = configs(graph.n, k)
    heads, trans = transitions(graph, k, cfg)
    states = np.empty(cfg.shape[0] * graph.n, dtype=np.uint8)
    row_ptr, col = graph.csr()
    col = np.ascontiguousarray(col if col.size else np.zeros(1, np.uint16))
    caps = ctypes.c_uint64(0)
    counts = np.zeros(max_passes, dtype=np.uint64)
    tr = trans if trans.size else np.zeros(1, np.uint64)
    passes = L.or_v2_solve(graph.n, _p(row_ptr, u32p), _p(col, u16p), k, p, _p(cfg, u16p),
                           cfg.shape[0], _p(heads, u64p), _p(tr, u64p), _p(states, u8p),
                           ctypes.byref(caps), _p(counts, u64p), max_passes, threads)
    if passes < 0:
        raise RuntimeError(f"oracle v2 failed ({passes})")
    sol = Solution(graph.n, k, p, 1, cfg, heads, trans, states, int(caps.value),
                   [int(x) for x in counts[:passes]])
    _verdict(sol)
    return sol


class SweepSample:
    """The CPU baseline's unit of work: one v1 pass (every column, k_cops_visibility.cpp:146-291)
    over a slice of the configurations, on a freshly initialised table."""

    def __init__(self, graph, k: int, p: int = 1):
        L = lib()
        self.graph, self.k, self.p = graph, k, p
        self.cfg = configs(graph.n, k)
        self.heads, self.trans = transitions(graph, k, self.cfg)
        self.row_ptr, col = graph.csr()
        self.col = np.ascontiguousarray(col if col.size else np.zeros(1, np.uint16))
        self.count = self.cfg.shape[0]
        self.states = np.empty(self.count * graph.n * 2 * p, dtype=np.uint8)
        L.or_v1_init(graph.n, k, p, _p(self.cfg, u16p), self.count, _p(self.states, u8p))

    @property
    def total_states(self) -> int:
        return self.count * self.graph.n * 2 * self.p

    def run(self, c0: int, c1: int, threads: int = 0) -> int:
        tr = self.trans if self.trans.size else np.zeros(1, np.uint64)
        return int(lib().or_v1_sweep_slice(self.graph.n, _p(self.row_ptr, u32p), _p(self.col, u16p), self.k,
                                           self.p, _p(self.heads, u64p), _p(tr, u64p), _p(self.states, u8p),
                                           c0, c1, threads))


def _verdict(sol: Solution) -> None:
    worst = ctypes.c_int(0)
    best = lib().or_verdict(sol.n, sol.configs.shape[0], sol.columns, _p(sol.states, u8p),
                            ctypes.byref(worst))
    sol.best_config = int(best)
    sol.capture_plies = int(worst.value)


def perfect_game(sol: Solution, graph) -> list:
    """util/perfect_game_extractor.py:67-165 restated over a two-column table: the positions
    (config id, robber) after each ply, the start first.  Empty for a LOSS."""
    if not sol.win:
        return []
    n, st, cfg = sol.n, sol.states, sol.configs
    rp, col = graph.csr()
    rnd = lambda c, r, t: int(st[(c * n + r) * 2 + t]) >> 1
    marked = lambda c, r, t: bool(st[(c * n + r) * 2 + t] & 1)
    holds = lambda c, r: r in set(int(x) for x in cfg[c])
    # robber start: first vertex with the largest column-0 round (:101-107)
    best_r, most = -1, -1
    for r in range(n):
        if rnd(sol.best_config, r, 0) > most:
            most, best_r = rnd(sol.best_config, r, 0), r
    c, r = sol.best_config, best_r
    out = [(c, r)]
    while len(out) < 4096:
        if holds(c, r):
            break
        nxt, low = c, 999                        # cops (:121-139)
        for t in range(int(sol.heads[c]), int(sol.heads[c + 1])):
            nc = int(sol.transitions[t]) // n
            if holds(nc, r):
                nxt = nc
                break
            if marked(nc, r, 1) and rnd(nc, r, 1) < low:
                low, nxt = rnd(nc, r, 1), nc
        c = nxt
        out.append((c, r))
        if holds(c, r):
            break
        nr, high = r, -1                         # robber (:147-160)
        for v in col[rp[r]:rp[r + 1]]:
            v = int(v)
            if marked(c, v, 0) and rnd(c, v, 0) > high:
                high, nr = rnd(c, v, 0), v
        r = nr
        out.append((c, r))
    return out


# ------------------------------------------------------------- reference binaries --------

RE_PASS = re.compile(r"Pass (\d+): Found (\d+) new winning states")
RE_CAPS = re.compile(r"Initialized (\d+) base captures")
RE_RESULT = re.compile(r"RESULT:\s+(WIN|LOSS)")
RE_POS = re.compile(r"Optimal Cop Start Positions:\s*\(([^)]*)\)")
RE_CAPTURE = re.compile(r"Capture Time:\s*(\d+)\s*plys")
RE_MAINLOOP = re.compile(r"Main Loop\s*-*=>\s*([\d.]+)\s*s")


def ref_available(name: str = "k_cops_visibility") -> bool:
    return os.path.exists(os.path.join(REF_DIR, name))


def read_table_file(path: str) -> dict:
    """Read the reference's 96-byte-header table file (lib/include/CacheManager.h:28-75)."""
    with open(path, "rb") as f:
        blob = f.read()
    h = struct.unpack("<12Q", blob[:96])
    k, n, cols, count, nstates, tsize, cs, rs, s1, s2, s3, s4 = h
    return {
        "k": k, "n": n, "columns": cols, "config_count": count, "num_states": nstates,
        "state_size": tsize, "cop_self": cs, "robber_self": rs,
        "configs": np.frombuffer(blob[s1:s2], dtype=np.uint8),
        "heads": np.frombuffer(blob[s2:s3], dtype=np.uint64),
        "transitions": np.frombuffer(blob[s3:s4], dtype=np.uint64),
        "states": np.frombuffer(blob[s4:], dtype=np.uint8),
        "raw": blob,
    }


def run_reference(matrix_path: str, k: int, p: int, solver: str = "k_cops_visibility",
                  timeout: float | None = None, keep_file: bool = True) -> dict:
    """Run a reference binary from a fresh working directory (so its table cache cannot hit)
    and return its parsed stdout plus, if keep_file, the table file it wrote."""
    exe = os.path.join(REF_DIR, solver)
    work = tempfile.mkdtemp(prefix="cr_ref_")
    try:
        src = os.path.abspath(matrix_path)
        dst = os.path.join(work, os.path.basename(src))
        shutil.copyfile(src, dst)
        proc = subprocess.run([exe, os.path.basename(dst), str(k), str(p)], cwd=work,
                              capture_output=True, text=True, timeout=timeout)
        out = proc.stdout
        res = {
            "stdout": out,
            "pass_counts": [int(b) for _, b in RE_PASS.findall(out)],
            "base_captures": int(RE_CAPS.search(out).group(1)) if RE_CAPS.search(out) else None,
            "result": RE_RESULT.search(out).group(1) if RE_RESULT.search(out) else None,
            "positions": RE_POS.search(out).group(1) if RE_POS.search(out) else "",
            "capture_plies": int(RE_CAPTURE.search(out).group(1)) if RE_CAPTURE.search(out) else None,
            "mainloop_s": float(RE_MAINLOOP.search(out).group(1)) if RE_MAINLOOP.search(out) else None,
        }
        if keep_file:
            cache = os.path.join(work, "cache")
            files = os.listdir(cache) if os.path.isdir(cache) else []
            res["table_file"] = files[0] if files else None
            res["table"] = read_table_file(os.path.join(cache, files[0])) if files else None
        return res
    finally:
        shutil.rmtree(work, ignore_errors=True)
