"""Serving: the solve server of the C ABI (cr_server_*) and the seeded request stream.

``Server`` wraps ``cr_server``: requests are submitted as they arrive, admitted by device
footprint as memory and workers free up, solved concurrently on per-worker streams, and their
tables stay resident until released.  ``request_stream`` draws the serving workload: a mix of
4-regular, Erdos-Renyi (mean degree 4) and Delaunay-thinned graphs with n log-uniform in
[20, 400], k uniform in {1, 2, 3}, 10% of requests with visibility period p in [2, 4] -- half
of those under the v1 rules (2p columns), half under the v2 macro-turn rules with k <= 2, p <= 3
and n <= 200 (the v2 search grows steeply with k, p and n: at k = 2, p = 4 or n = 400 one solve
takes seconds to minutes) -- and Poisson arrival times at a given rate.  ``run_stream``
replays it.
"""
from __future__ import annotations

import ctypes
import threading
import time
from dataclasses import dataclass

import numpy as np

from . import graphs as G
from . import native as N


class Server:
    def __init__(self, device: int = 0, memory_budget: int = 0, workers: int = 8):
        self.ptr = ctypes.c_void_p()
        rc = N.lib().cr_server_create(device, memory_budget, workers, ctypes.byref(self.ptr))
        if rc:
            raise N.CrGpuError(rc, "cr_server_create failed")
        self._keep = {}

    def submit(self, graph: G.Graph, k: int, p: int = 1, rules: int = N.CR_RULES_V1) -> int:
        row_ptr, col = graph.csr()
        if col.size == 0:
            col = np.zeros(1, dtype=np.uint16)
        cg = N.CrGraph(graph.n, row_ptr.ctypes.data_as(N.c_u32p), col.ctypes.data_as(N.c_u16p))
        rid = ctypes.c_uint64()
        rc = N.lib().cr_server_submit(self.ptr, ctypes.byref(cg), k, p, rules, ctypes.byref(rid))
        if rc:
            raise N.CrGpuError(rc, N.lib().cr_server_last_error(self.ptr).decode())
        return int(rid.value)

    def poll(self, rid: int, wait_ms: int = 0) -> dict | None:
        r = N.CrRequestResult()
        rc = N.lib().cr_server_poll(self.ptr, rid, wait_ms, ctypes.byref(r))
        if rc == 8:  # CR_ERR_STATE: still queued or running
            return None
        if rc:
            raise N.CrGpuError(rc, N.lib().cr_server_last_error(self.ptr).decode())
        return {f: getattr(r, f) for f, _ in N.CrRequestResult._fields_}

    def read_states(self, rid: int, nbytes: int) -> np.ndarray:
        out = np.empty(nbytes, dtype=np.uint8)
        rc = N.lib().cr_server_read_states(self.ptr, rid, out.ctypes.data_as(N.c_u8p), nbytes)
        if rc:
            raise N.CrGpuError(rc, "cr_server_read_states")
        return out

    def release(self, rid: int) -> None:
        rc = N.lib().cr_server_release(self.ptr, rid)
        if rc:
            raise N.CrGpuError(rc, "cr_server_release")

    def stats(self) -> dict:
        s = N.CrServerStats()
        N.lib().cr_server_stats(self.ptr, ctypes.byref(s))
        return {f: getattr(s, f) for f, _ in N.CrServerStats._fields_}

    def close(self) -> None:
        if self.ptr:
            N.lib().cr_server_destroy(self.ptr)
            self.ptr = ctypes.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()


@dataclass
class Request:
    graph: G.Graph
    k: int
    p: int
    kind: str
    arrival_s: float
    rules: int = N.CR_RULES_V1


def _delaunay_fast(n: int, seed: int, mean_degree: float = 4.5) -> G.Graph:
    """Delaunay triangulation of n uniform points thinned at random to a mean degree while
    connected: a random spanning tree of the triangulation is kept and random other edges are
    dropped (no connectivity test needed)."""
    from scipy.spatial import Delaunay

    rng = np.random.default_rng(seed)
    pts = rng.random((n, 2))
    tri = Delaunay(pts)
    e = np.concatenate([tri.simplices[:, [0, 1]], tri.simplices[:, [1, 2]], tri.simplices[:, [2, 0]]])
    e = np.unique(np.sort(e, axis=1), axis=0)
    order = rng.permutation(len(e))
    parent = np.arange(n)

    def find(x):
        while parent[x] != x:
            parent[x] = parent[parent[x]]
            x = parent[x]
        return x

    tree, rest = [], []
    for i in order:
        a, b = find(e[i, 0]), find(e[i, 1])
        if a != b:
            parent[a] = b
            tree.append(i)
        else:
            rest.append(i)
    keep = max(0, int(round(mean_degree * n / 2)) - len(tree))
    chosen = np.array(tree + rest[:keep], dtype=np.int64)
    adj = np.zeros((n, n), dtype=np.uint8)
    adj[e[chosen, 0], e[chosen, 1]] = 1
    adj[e[chosen, 1], e[chosen, 0]] = 1
    return G.Graph(adj)


def _er_connected_fast(n: int, mean_degree: float, seed: int) -> G.Graph:
    """G(n, p) with p = mean_degree / (n - 1), made connected by joining every other
    component to the largest one with one random edge (a sparse G(n, p) is rarely connected,
    so redrawing until it is would take thousands of draws at n = 400)."""
    from scipy.sparse.csgraph import connected_components

    rng = np.random.default_rng(seed)
    p = min(1.0, mean_degree / max(n - 1, 1))
    iu = np.triu_indices(n, 1)
    pick = rng.random(iu[0].size) < p
    adj = np.zeros((n, n), dtype=np.uint8)
    adj[iu[0][pick], iu[1][pick]] = 1
    adj = adj | adj.T
    ncomp, label = connected_components(adj, directed=False)
    if ncomp > 1:
        big = np.bincount(label).argmax()
        big_nodes = np.flatnonzero(label == big)
        for c in range(ncomp):
            if c == big:
                continue
            u = rng.choice(np.flatnonzero(label == c))
            v = rng.choice(big_nodes)
            adj[u, v] = adj[v, u] = 1
    return G.Graph(adj)


def request_stream(count: int, rate_per_s: float, seed: int = 7, n_lo: int = 20, n_hi: int = 400,
                   p_share: float = 0.10, v2_share: float = 0.5) -> list:
    """The seeded serving workload (graphs, k, p, rules and Poisson arrival times).  A share
    p_share of the requests has a visibility period p in [2, 4]; v2_share of those use the v2
    rules (drawn from a second seeded stream, so the rest of the workload is unchanged)."""
    rng = np.random.default_rng(seed)
    vrng = np.random.default_rng(seed ^ 0x5EED)
    gaps = rng.exponential(1.0 / rate_per_s, size=count)
    arrivals = np.cumsum(gaps) - gaps[0]
    out = []
    for i in range(count):
        n = int(round(np.exp(rng.uniform(np.log(n_lo), np.log(n_hi)))))
        kind = ("regular4", "er4", "delaunay")[int(rng.integers(0, 3))]
        k = int(rng.integers(1, 4))
        p = int(rng.integers(2, 5)) if rng.random() < p_share else 1
        rules = N.CR_RULES_V1
        if p > 1 and vrng.random() < v2_share:
            # v2 requests stay where the macro-turn search takes at most about 0.1 s on this GPU
            # (Delaunay n = 200, k = 2, p = 3); p = 4 or n = 400 at k = 2 run for seconds to minutes
            rules = N.CR_RULES_V2
            k, p, n = min(k, 2), min(p, 3), min(n, 200)
        gs = G.sub_seed(seed, i) & 0xFFFFFFFF
        if kind == "regular4":
            g = G.regular4(n + (n % 2), gs)
        elif kind == "er4":
            g = _er_connected_fast(n, 4.0, gs)
        else:
            g = _delaunay_fast(n, gs)
        out.append(Request(g, k, p, kind, float(arrivals[i]), rules))
    return out


def run_stream(server: Server, reqs: list, release: bool = True) -> dict:
    """Replay requests at their arrival times; returns latencies and totals."""
    ids = [None] * len(reqs)
    done = [None] * len(reqs)
    t0 = time.perf_counter()

    def submitter():
        for i, r in enumerate(reqs):
            delay = r.arrival_s - (time.perf_counter() - t0)
            if delay > 0:
                time.sleep(delay)
            ids[i] = server.submit(r.graph, r.k, r.p, r.rules)

    th = threading.Thread(target=submitter)
    th.start()
    pending = 0
    while pending < len(reqs):
        if ids[pending] is None:
            time.sleep(0.0005)
            continue
        res = server.poll(ids[pending], wait_ms=-1)
        done[pending] = res
        if release:
            server.release(ids[pending])
        pending += 1
    th.join()
    wall = time.perf_counter() - t0
    lat = np.array([d["latency_ms"] for d in done])
    states = sum(int(d["states"]) for d in done)
    return {"requests": len(reqs), "wall_s": wall, "p50_ms": float(np.percentile(lat, 50)),
            "p99_ms": float(np.percentile(lat, 99)), "mean_ms": float(lat.mean()),
            "states": states, "states_per_s": states / wall, "results": done, "ids": ids,
            "stats": server.stats()}
