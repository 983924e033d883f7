"""Failure paths: bad input is refused with an error code and a message, phases out of order
are refused, and the context stays usable afterwards."""
import ctypes

import numpy as np
import pytest

from copsandrobbers_gb300 import graphs as G
from copsandrobbers_gb300 import native as N
from copsandrobbers_gb300.solver import Solver, solve

pytestmark = pytest.mark.gpu


def test_bad_arguments(gpu_ctx):
    g = G.regular4(12, 1)
    for k, p, rules, code in [(0, 1, 1, 4),
                              (5, 1, 1, 4), (2, 0, 1, 1), (2, 1, 7, 1)]:
        with pytest.raises(N.CrGpuError) as e:
            Solver(gpu_ctx, g, k, p, rules)
        assert e.value.code == code


def test_empty_graph_refused(gpu_ctx):
    with pytest.raises(N.CrGpuError) as e:
        Solver(gpu_ctx, G.Graph(np.zeros((0, 0), np.uint8)), 1, 1)
    assert e.value.code == 1 and "empty" in str(e.value)


def test_neighbour_out_of_range_refused(gpu_ctx):
    rp = np.array([0, 1, 2], dtype=np.uint32)
    col = np.array([1, 7], dtype=np.uint16)
    g = N.CrGraph(2, rp.ctypes.data_as(N.c_u32p), col.ctypes.data_as(N.c_u16p))
    out = ctypes.c_void_p()
    rc = N.lib().cr_solver_create(gpu_ctx.ptr, ctypes.byref(g), 1, 1, 1, ctypes.byref(out))
    assert rc == 1


def test_phase_order_enforced(gpu_ctx):
    with Solver(gpu_ctx, G.regular4(12, 1), 2, 1) as s:
        with pytest.raises(N.CrGpuError) as e:
            s.step()
        assert e.value.code == 8
    # the context still works
    r = solve(gpu_ctx, G.regular4(12, 1), 1, 1)
    assert r.pass_counts[-1] == 0


def test_buffer_too_small(gpu_ctx):
    with Solver(gpu_ctx, G.regular4(12, 1), 2, 1) as s:
        s.init(); s.run()
        buf = np.zeros(10, dtype=np.uint8)
        rc = N.lib().cr_solver_read_states(s.ptr, buf.ctypes.data_as(N.c_u8p), buf.size)
        assert rc == 1
