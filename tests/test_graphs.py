"""Graph input: the matrix parser's edge cases and the seeded generators."""
import numpy as np
import pytest

from copsandrobbers_gb300 import graphs as G


def test_parse_roundtrip():
    g = G.regular4(20, 1)
    assert np.array_equal(G.parse_matrix(G.format_matrix(g)).adj, g.adj)


@pytest.mark.parametrize("text,n,edges", [
    (b"010\n101\n010\n-", 3, {(0, 1), (1, 0), (1, 2), (2, 1)}),
    (b"010\r\n101\r\n010\r\n-", 3, {(0, 1), (1, 0), (1, 2), (2, 1)}),   # '\r' is skipped
    (b"01\n10", 2, {(0, 1), (1, 0)}),                                  # no end marker
    (b"01\n\n\n10\n-", 2, {(0, 1), (1, 0)}),                          # blank lines do not advance
    (b"0 1\n1 0\n-", 3, {(0, 1), (1, 0)}),                             # width counts every char
    (b"011\n1-11\n110", 3, {(0, 1), (0, 2), (1, 0)}),                  # '-' ends the matrix
    (b"-", 0, set()),
    (b"", 0, set()),
])
def test_parse_edge_cases(text, n, edges):
    g = G.parse_matrix(text)
    assert g.n == n
    assert {(int(a), int(b)) for a, b in zip(*np.nonzero(g.adj))} == edges


def test_regular4_properties():
    for n, seed in ((16, 3), (255, 12345), (256, 12345)):
        g = G.regular4(n, seed)
        assert g.n == n
        assert (g.adj.sum(axis=1) == 4).all()
        assert (g.adj == g.adj.T).all() and not g.adj.diagonal().any()
        assert G.is_connected(g.adj)
    assert G.regular4(64, 9).digest() == G.regular4(64, 9).digest()


def test_committed_synthetic_graphs_regenerate():
    import os
    here = os.path.join(os.path.dirname(__file__), "golden", "graphs")
    for n in (255, 256):
        assert np.array_equal(G.load_matrix(os.path.join(here, f"regular4_n{n}_s12345.txt")).adj,
                              G.regular4(n, 12345).adj)
    d = G.load_matrix(os.path.join(here, "delaunay_n199_s2024.txt"))
    assert np.array_equal(d.adj, G.delaunay_thinned(199, 2024).adj)
    assert abs(d.mean_degree() - 4.5) < 0.05 and G.is_connected(d.adj)


def test_erdos_renyi_properties():
    g = G.erdos_renyi(40, 4.0, 11)
    assert G.is_connected(g.adj) and (g.adj == g.adj.T).all() and not g.adj.diagonal().any()
