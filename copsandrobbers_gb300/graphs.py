"""Graph input: the reference's adjacency-matrix text format and seeded generators.

Text format (lib/src/Graph.cpp:15-79 of the reference): one row of '0'/'1' characters per
vertex, rows separated by '\\n', the file ended by '-'.  The vertex count is the width of the
first line (up to the first '\\n', '\\r' or '-', Graph.cpp:26-30).  Any other character is
skipped; a '\\n' only advances the row when the current row already holds a digit
(Graph.cpp:63-68).  Neighbour lists are the set columns of each row in increasing order
(lib/src/AdjacencyList.cpp:33-76), which is the order every solver iterates them in.

The generators produce the seeded synthetic workloads the benchmarks are quoted on (no public
dataset exists for this path):

* ``regular4``   - connected 4-regular graph from the configuration model, rejecting draws
                   with loops or multi-edges (the large single solve, n=256 and its n=255 twin).
* ``erdos_renyi`` - connected G(n, p) with p chosen for a target mean degree (batched work).
* ``delaunay_thinned`` - Delaunay triangulation of uniform points in the unit square, edges
                   dropped at random while keeping connectivity down to a mean degree
                   (limited-visibility work).
"""
from __future__ import annotations

import hashlib
import os
from dataclasses import dataclass

import numpy as np

__all__ = [
    "Graph", "parse_matrix", "load_matrix", "format_matrix", "save_matrix",
    "regular4", "erdos_renyi", "delaunay_thinned", "is_connected", "sub_seed",
]


@dataclass
class Graph:
    """A directed 0/1 adjacency matrix as the reference reads it (row v = out-edges of v)."""

    adj: np.ndarray  # uint8 [n, n]

    @property
    def n(self) -> int:
        return int(self.adj.shape[0])

    def neighbours(self, v: int) -> np.ndarray:
        return np.flatnonzero(self.adj[v]).astype(np.int32)

    def csr(self) -> tuple[np.ndarray, np.ndarray]:
        """Row pointers (uint32) and column indices (uint16) in increasing column order."""
        deg = self.adj.sum(axis=1, dtype=np.int64)
        row_ptr = np.zeros(self.n + 1, dtype=np.uint32)
        np.cumsum(deg, out=row_ptr[1:])
        col = np.nonzero(self.adj)[1].astype(np.uint16)  # row-major order == per-row ascending
        return row_ptr, col

    def max_degree(self) -> int:
        return int(self.adj.sum(axis=1).max()) if self.n else 0

    def mean_degree(self) -> float:
        return float(self.adj.sum()) / max(self.n, 1)

    def digest(self) -> str:
        return hashlib.sha256(np.ascontiguousarray(self.adj).tobytes()).hexdigest()[:16]


def parse_matrix(data: bytes) -> Graph:
    """Parse matrix text exactly as Graph::Graph does (lib/src/Graph.cpp:15-79).

    Returns an empty (n=0) graph where the reference would leave nodeCount at 0.
    """
    if isinstance(data, str):
        data = data.encode()
    n = 0
    while n < len(data) and data[n] not in (0x0A, 0x0D, 0x2D):
        n += 1
    adj = np.zeros((n, n), dtype=np.uint8)
    if n == 0:
        return Graph(adj)
    row = col = 0
    for ch in data:
        if ch == 0x2D:  # '-'
            break
        if ch == 0x30 or ch == 0x31:  # '0' / '1'
            if row < n and col < n:
                adj[row, col] = ch - 0x30
            col += 1
        elif ch == 0x0A and col > 0:
            row += 1
            col = 0
    return Graph(adj)


def load_matrix(path: str | os.PathLike) -> Graph:
    with open(path, "rb") as f:
        return parse_matrix(f.read())


def format_matrix(g: Graph) -> bytes:
    rows = [bytes((0x30 + int(x)) for x in g.adj[i]) for i in range(g.n)]
    return b"\n".join(rows) + b"\n-"


def save_matrix(g: Graph, path: str | os.PathLike) -> None:
    with open(path, "wb") as f:
        f.write(format_matrix(g))


def is_connected(adj: np.ndarray) -> bool:
    n = adj.shape[0]
    if n == 0:
        return False
    seen = np.zeros(n, dtype=bool)
    seen[0] = True
    stack = [0]
    while stack:
        v = stack.pop()
        for u in np.flatnonzero(adj[v]):
            if not seen[u]:
                seen[u] = True
                stack.append(int(u))
    return bool(seen.all())


def sub_seed(master: int, index: int) -> int:
    """Per-graph seed = hash(master, index), stable across platforms."""
    h = hashlib.sha256(f"{master}:{index}".encode()).digest()
    return int.from_bytes(h[:8], "little")


def regular4(n: int, seed: int, degree: int = 4) -> Graph:
    """Connected `degree`-regular simple graph by the configuration model with rejection."""
    if (n * degree) % 2:
        raise ValueError("n * degree must be even")
    rng = np.random.default_rng(seed)
    stubs = np.repeat(np.arange(n, dtype=np.int64), degree)
    for _ in range(100000):
        perm = rng.permutation(stubs)
        a, b = perm[0::2], perm[1::2]
        if np.any(a == b):
            continue
        lo, hi = np.minimum(a, b), np.maximum(a, b)
        key = lo * n + hi
        if np.unique(key).size != key.size:
            continue
        adj = np.zeros((n, n), dtype=np.uint8)
        adj[a, b] = 1
        adj[b, a] = 1
        if is_connected(adj):
            return Graph(adj)
    raise RuntimeError("configuration model did not produce a simple connected graph")


def erdos_renyi(n: int, mean_degree: float, seed: int) -> Graph:
    """Connected G(n, p) with p = mean_degree / (n - 1); disconnected draws are redrawn."""
    rng = np.random.default_rng(seed)
    p = min(1.0, mean_degree / max(n - 1, 1))
    iu = np.triu_indices(n, 1)
    for _ in range(100000):
        pick = rng.random(iu[0].size) < p
        adj = np.zeros((n, n), dtype=np.uint8)
        adj[iu[0][pick], iu[1][pick]] = 1
        adj = adj | adj.T
        if is_connected(adj):
            return Graph(adj)
    raise RuntimeError("G(n, p) draws stayed disconnected")


def delaunay_thinned(n: int, seed: int, mean_degree: float = 4.5) -> Graph:
    """Delaunay triangulation of n uniform points, randomly thinned while connected."""
    from scipy.spatial import Delaunay

    rng = np.random.default_rng(seed)
    pts = rng.random((n, 2))
    tri = Delaunay(pts)
    edges = set()
    for s in tri.simplices:
        for i in range(3):
            u, v = int(s[i]), int(s[(i + 1) % 3])
            edges.add((min(u, v), max(u, v)))
    edges = sorted(edges)
    adj = np.zeros((n, n), dtype=np.uint8)
    for u, v in edges:
        adj[u, v] = adj[v, u] = 1
    target = int(round(mean_degree * n / 2))
    order = rng.permutation(len(edges))
    count = len(edges)
    for idx in order:
        if count <= target:
            break
        u, v = edges[idx]
        adj[u, v] = adj[v, u] = 0
        if is_connected(adj):
            count -= 1
        else:
            adj[u, v] = adj[v, u] = 1
    return Graph(adj)
