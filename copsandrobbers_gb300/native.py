"""ctypes binding of libcrgpu.so (the C ABI declared in include/crgpu.h).

The library is the only compute path: if it is missing or fails to load, every entry point
raises instead of falling back to anything else.
"""
from __future__ import annotations

import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libcrgpu.so")

CR_OK = 0
ERRORS = {
    1: "CR_ERR_INVALID", 2: "CR_ERR_NOMEM", 3: "CR_ERR_CUDA", 4: "CR_ERR_LIMIT",
    5: "CR_ERR_INTERNAL", 6: "CR_ERR_BUDGET", 7: "CR_ERR_IO", 8: "CR_ERR_STATE",
}
CR_RULES_V1 = 1
CR_RULES_V2 = 2
CR_COP_STAY = 0x10
# kernel forms of a v1 solve (cr_solver_set_forms)
CR_FORM_FUSED_FIRST = 0x01
CR_FORM_PUSH = 0x02
CR_FORM_PULL = 0x04
CR_FORM_SEPARABLE = 0x08
CR_FORM_FRESH_LAST = 0x10
CR_FORMS_ALL = 0x1F
CR_ROBBER_STAY = 0x20
CR_MAX_K = 4

c_u64p = ctypes.POINTER(ctypes.c_uint64)
c_u32p = ctypes.POINTER(ctypes.c_uint32)
c_u16p = ctypes.POINTER(ctypes.c_uint16)
c_u8p = ctypes.POINTER(ctypes.c_uint8)
c_i32p = ctypes.POINTER(ctypes.c_int32)


class CrGraph(ctypes.Structure):
    _fields_ = [("n", ctypes.c_int32), ("row_ptr", c_u32p), ("col_idx", c_u16p)]


class CrVerdict(ctypes.Structure):
    _fields_ = [("win", ctypes.c_int32), ("capture_plies", ctypes.c_int32),
                ("best_config", ctypes.c_int64), ("positions", ctypes.c_uint16 * CR_MAX_K)]


class CrTableSizes(ctypes.Structure):
    _fields_ = [("config_count", ctypes.c_uint64), ("num_states", ctypes.c_uint64),
                ("columns", ctypes.c_int32), ("k", ctypes.c_int32), ("n", ctypes.c_int32),
                ("pad", ctypes.c_int32), ("transitions", ctypes.c_uint64)]


class CrSolveStats(ctypes.Structure):
    _fields_ = [("init_ms", ctypes.c_double), ("main_ms", ctypes.c_double),
                ("cop_step_ms", ctypes.c_double), ("cop_step_launches", ctypes.c_int64),
                ("kernel_launches", ctypes.c_int64), ("passes", ctypes.c_int32),
                ("slots", ctypes.c_int32), ("resolved", ctypes.c_uint64)]


class CrV2HashStats(ctypes.Structure):
    _fields_ = [(f, ctypes.c_uint64) for f in ("capacity", "child_visits", "entries", "fills")]


class CrBatchResult(ctypes.Structure):
    _fields_ = [("solved", ctypes.c_int32), ("status", ctypes.c_int32), ("win", ctypes.c_int32),
                ("capture_plies", ctypes.c_int32), ("passes", ctypes.c_int32), ("pad", ctypes.c_int32),
                ("best_config", ctypes.c_int64), ("base_captures", ctypes.c_uint64),
                ("states", ctypes.c_uint64), ("digest", ctypes.c_uint64), ("pass_hash", ctypes.c_uint64)]


class CrBatchStats(ctypes.Structure):
    _fields_ = [("ms", ctypes.c_double), ("states", ctypes.c_uint64), ("ctas", ctypes.c_int32),
                ("threads", ctypes.c_int32), ("slot_bytes", ctypes.c_int64), ("busy_frac", ctypes.c_double),
                ("tail_ms", ctypes.c_double)]


class CrRequestResult(ctypes.Structure):
    _fields_ = [("status", ctypes.c_int32), ("win", ctypes.c_int32), ("capture_plies", ctypes.c_int32),
                ("passes", ctypes.c_int32), ("best_config", ctypes.c_int64), ("base_captures", ctypes.c_uint64),
                ("states", ctypes.c_uint64), ("digest", ctypes.c_uint64), ("pass_hash", ctypes.c_uint64),
                ("queue_ms", ctypes.c_double), ("run_ms", ctypes.c_double), ("latency_ms", ctypes.c_double)]


class CrServerStats(ctypes.Structure):
    _fields_ = [(f, ctypes.c_uint64) for f in ("completed", "failed", "queued", "running", "max_running",
                                               "memory_budget", "memory_in_use", "peak_memory_in_use",
                                               "states_done")] + [("busy_ms", ctypes.c_double)]


class CrGpuError(RuntimeError):
    def __init__(self, code: int, message: str):
        super().__init__(f"{ERRORS.get(code, code)}: {message}")
        self.code = code


# Every symbol include/crgpu.h declares, with (restype, argtypes).
SIGNATURES = {
    "cr_context_create": (ctypes.c_int, [ctypes.c_int32, ctypes.c_void_p, ctypes.POINTER(ctypes.c_void_p)]),
    "cr_context_destroy": (ctypes.c_int, [ctypes.c_void_p]),
    "cr_context_last_error": (ctypes.c_char_p, [ctypes.c_void_p]),
    "cr_context_set_profiling": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int32]),
    "cr_context_set_cache_limit": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_uint64]),
    "cr_solver_footprint": (ctypes.c_uint64, [ctypes.c_int32, ctypes.c_int32, ctypes.c_int32, ctypes.c_int32]),
    "cr_graph_parse": (ctypes.c_int, [ctypes.c_char_p, ctypes.c_size_t, c_i32p, c_u32p, c_u16p,
                                      ctypes.c_size_t, ctypes.POINTER(ctypes.c_size_t)]),
    "cr_solver_create": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(CrGraph), ctypes.c_int32,
                                        ctypes.c_int32, ctypes.c_int32, ctypes.POINTER(ctypes.c_void_p)]),
    "cr_solver_destroy": (ctypes.c_int, [ctypes.c_void_p]),
    "cr_solver_init": (ctypes.c_int, [ctypes.c_void_p, c_u64p]),
    "cr_solver_pass": (ctypes.c_int, [ctypes.c_void_p, c_u64p]),
    "cr_solver_run": (ctypes.c_int, [ctypes.c_void_p, c_u64p, ctypes.c_int32, c_i32p]),
    "cr_solver_verdict": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(CrVerdict)]),
    "cr_solver_sizes": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(CrTableSizes)]),
    "cr_solver_stats": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(CrSolveStats)]),
    "cr_solver_read_states": (ctypes.c_int, [ctypes.c_void_p, c_u8p, ctypes.c_size_t]),
    "cr_solver_device_states": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_void_p),
                                               ctypes.POINTER(ctypes.c_size_t)]),
    "cr_solver_read_configs": (ctypes.c_int, [ctypes.c_void_p, c_u8p, ctypes.c_size_t]),
    "cr_solver_build_transitions": (ctypes.c_int, [ctypes.c_void_p, c_u64p]),
    "cr_solver_read_transitions": (ctypes.c_int, [ctypes.c_void_p, c_u64p, ctypes.c_size_t, c_u64p,
                                                  ctypes.c_size_t]),
    "cr_solver_write_table_file": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_char_p]),
    "cr_solve": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(CrGraph), ctypes.c_int32, ctypes.c_int32,
                                ctypes.c_int32, c_u8p, ctypes.c_size_t, c_u64p, ctypes.c_int32, c_i32p,
                                ctypes.POINTER(CrVerdict), ctypes.POINTER(CrSolveStats)]),
    "cr_batch_solve": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(CrGraph), ctypes.c_int32, ctypes.c_int32,
                                      ctypes.c_int32, ctypes.c_int32, c_i32p, ctypes.POINTER(CrBatchResult),
                                      ctypes.POINTER(CrBatchStats)]),
    "cr_solver_digest": (ctypes.c_int, [ctypes.c_void_p, c_u64p]),
    "cr_solver_load_table_file": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_char_p]),
    "cr_solver_v2_hash_stats": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(CrV2HashStats)]),
    "cr_solver_set_v2_hash_capacity": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_uint64]),
    "cr_solver_set_forms": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_uint32]),
    "cr_solver_perfect_game": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_int64),
                                              ctypes.POINTER(ctypes.c_int32), ctypes.c_int32,
                                              ctypes.POINTER(ctypes.c_int32), ctypes.POINTER(ctypes.c_int32)]),
    "cr_server_create": (ctypes.c_int, [ctypes.c_int32, ctypes.c_uint64, ctypes.c_int32, ctypes.POINTER(ctypes.c_void_p)]),
    "cr_server_submit": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(CrGraph), ctypes.c_int32, ctypes.c_int32,
                                        ctypes.c_int32, c_u64p]),
    "cr_server_poll": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_uint64, ctypes.c_int32, ctypes.POINTER(CrRequestResult)]),
    "cr_server_read_states": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_uint64, c_u8p, ctypes.c_size_t]),
    "cr_server_release": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_uint64]),
    "cr_server_stats": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(CrServerStats)]),
    "cr_server_last_error": (ctypes.c_char_p, [ctypes.c_void_p]),
    "cr_server_destroy": (ctypes.c_int, [ctypes.c_void_p]),
    "cr_solve_v1_noalloc": (ctypes.c_int, [ctypes.POINTER(CrGraph), ctypes.c_int32, ctypes.c_int32,
                                           ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t, c_u64p,
                                           ctypes.c_int32, c_i32p, c_u64p, ctypes.c_char_p, ctypes.c_size_t]),
}

_lib = None


def lib():
    """Load libcrgpu.so (raising if it is absent: there is no other compute path)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError(f"{LIB_PATH} is missing: run __graft_entry__.build() (or python -m "
                              "copsandrobbers_gb300.build) to compile the CUDA extension")
        L = ctypes.CDLL(LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


MASK64 = (1 << 64) - 1


def mix64(z: int) -> int:
    """splitmix64 finaliser (the mixer of the table digest)."""
    z &= MASK64
    z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & MASK64
    z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & MASK64
    return z ^ (z >> 31)


def table_digest(table) -> int:
    """The digest cr_solver_digest computes, restated with numpy (tables of any length)."""
    import numpy as np

    b = np.ascontiguousarray(table, dtype=np.uint8).ravel()
    pad = (-b.size) % 8
    if pad:
        b = np.concatenate([b, np.zeros(pad, np.uint8)])
    w = b.view("<u8").astype(np.uint64)
    j = np.arange(w.size, dtype=np.uint64)
    with np.errstate(over="ignore"):
        z = w ^ (j * np.uint64(0x9E3779B97F4A7C15))
        z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
        z = z ^ (z >> np.uint64(31))
        return int(z.sum(dtype=np.uint64))


def pass_hash(counts) -> int:
    """The pass-count hash of a batch result: sum_i mix64(count_i ^ (i * 0xD1B54A32D192ED03))."""
    h = 0
    for i, c in enumerate(counts, start=1):
        h = (h + mix64(int(c) ^ ((i * 0xD1B54A32D192ED03) & MASK64))) & MASK64
    return h


def declared_symbols() -> list[str]:
    """Function names declared in include/crgpu.h and include/*.h, parsed from the headers."""
    import glob
    import re

    names = []
    for h in sorted(glob.glob(os.path.join(os.path.dirname(HERE), "include", "*.h"))):
        text = open(h).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        names += re.findall(r"^\s*(?:const\s+)?[A-Za-z_][A-Za-z0-9_]*\s*\*?\s*(cr_[a-z0-9_]+)\s*\(", text, flags=re.M)
    return sorted(set(names))
