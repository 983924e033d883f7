"""The allocation-free entry point, cr_solve_v1_noalloc, against the allocating one.

Callers that cannot allocate memory (a pool or budget they do not own, a path that must not
take the allocator's locks, an embedder that forbids library-owned device memory) pass their
own device table and the library works inside a fixed 64 MiB area of its own image.  This
file is collected last so that a run stopping at the first failure has already run the rest.
Each case calls the entry point twice in a row -- the scratch area keeps the previous call's
contents, which must not leak into the next -- and compares both tables and pass counts with
cr_solve, bit for bit (the tables are integers: no tolerance)."""
import ctypes

import numpy as np
import pytest

from copsandrobbers_gb300 import graphs as G
from copsandrobbers_gb300 import native as N
from copsandrobbers_gb300.solver import Context, solve

pytestmark = pytest.mark.gpu


def _noalloc(graph, k, p, states_dev, nbytes):
    L = N.lib()
    row_ptr, col = graph.csr()
    if col.size == 0:
        col = np.zeros(1, dtype=np.uint16)
    cg = N.CrGraph(graph.n, row_ptr.ctypes.data_as(N.c_u32p), col.ctypes.data_as(N.c_u16p))
    counts = np.zeros(4096, dtype=np.uint64)
    passes = ctypes.c_int32()
    caps = ctypes.c_uint64()
    err = ctypes.create_string_buffer(256)
    rc = L.cr_solve_v1_noalloc(ctypes.byref(cg), k, p, None, ctypes.c_void_p(states_dev), nbytes,
                               counts.ctypes.data_as(N.c_u64p), counts.size, ctypes.byref(passes),
                               ctypes.byref(caps), err, len(err))
    return rc, [int(x) for x in counts[: passes.value]], int(caps.value), err.value.decode()


@pytest.mark.parametrize("name,graph,k,p", [
    ("petersen", G.parse_matrix(open(__file__.replace("test_zz_no_alloc.py", "golden/matrices/peterson.txt"), "rb").read()), 3, 1),
    ("er40", G.erdos_renyi(40, 4.0, 7), 2, 2),
    ("regular64", G.regular4(64, 3), 3, 1),
    ("er24-p3", G.erdos_renyi(24, 3.0, 11), 3, 3),
])
def test_noalloc_matches_allocating_solve(name, graph, k, p):
    torch = pytest.importorskip("torch")
    with Context(0) as ctx:
        ref = solve(ctx, graph, k, p)
    nbytes = ref.states.size
    for call in range(2):
        out = torch.full((nbytes,), 0x55, dtype=torch.uint8, device="cuda")
        rc, counts, caps, msg = _noalloc(graph, k, p, out.data_ptr(), nbytes)
        assert rc == 0, msg
        torch.cuda.synchronize()
        got = out.cpu().numpy()
        assert counts == ref.pass_counts, (name, call)
        assert caps == ref.base_captures
        assert np.array_equal(got, ref.states), (name, call)


def test_noalloc_refuses_oversized_solve():
    torch = pytest.importorskip("torch")
    g = G.regular4(256, 12345)
    out = torch.empty(16, dtype=torch.uint8, device="cuda")
    rc, _, _, msg = _noalloc(g, 3, 1, out.data_ptr(), 1 << 40)
    assert rc == 4
    assert "scratch" in msg and "64 MiB" in msg
