"""The C-ABI library loads and exports every symbol include/*.h declares; host-only entry
points (parsing, footprint) agree with the Python restatements.  No GPU compute here."""
import glob
import os

import numpy as np
import pytest

from copsandrobbers_gb300 import graphs as G
from copsandrobbers_gb300 import native as N
from copsandrobbers_gb300.solver import footprint, parse_matrix

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_every_declared_symbol_is_exported():
    L = N.lib()
    declared = N.declared_symbols()
    assert len(declared) >= 20
    missing = [s for s in declared if not hasattr(L, s)]
    assert not missing, missing
    # and the binding knows every one of them
    assert set(declared) <= set(N.SIGNATURES), set(declared) - set(N.SIGNATURES)


@pytest.mark.parametrize("path", sorted(glob.glob(os.path.join(ROOT, "tests", "golden", "matrices", "*.txt")))
                         + sorted(glob.glob(os.path.join(ROOT, "tests", "golden", "graphs", "*.txt"))))
def test_library_parser_matches_reference_semantics(path):
    data = open(path, "rb").read()
    assert np.array_equal(parse_matrix(data).adj, G.parse_matrix(data).adj)


@pytest.mark.parametrize("text", [b"010\r\n101\r\n010\r\n-", b"01\n\n\n10\n-", b"0 1\n1 0\n-",
                                  b"011\n1-11\n110", b"-", b"1"])
def test_library_parser_edge_cases(text):
    assert np.array_equal(parse_matrix(text).adj, G.parse_matrix(text).adj)


def test_footprint_scales():
    small, large = footprint(10, 3), footprint(256, 3)
    assert 0 < small < large
    # table bytes alone: C(258,3) * 256 * 2
    assert large > 2_829_056 * 256 * 2
    assert footprint(256, 3, 2) > large                      # 4 columns instead of 2
    assert footprint(199, 2, 3, N.CR_RULES_V2) > 0
    assert footprint(0, 3) == 0


def test_footprint_counts_pair_rows_and_cloud_table():
    # k = 3: the separable cop turn's pair rows, P * n rows of S * rwp words (P = n(n+1)/2)
    table_128 = 357_760 * 128 * 2
    pair_rows_128 = 128 * 129 // 2 * 128 * 2 * 4 * 4
    assert footprint(128, 3) > table_128 + pair_rows_128
    # v2 with p >= 3 holds the cloud table: 2^23 slots of an 8-byte key word (key and value) and
    # a 4 * rwp-byte cloud at n = 199, k = 2
    assert footprint(199, 2, 3, N.CR_RULES_V2) - footprint(199, 2, 2, N.CR_RULES_V2) == (1 << 23) * (8 + 4 * 8)


def test_missing_library_fails_loudly(monkeypatch, tmp_path):
    monkeypatch.setattr(N, "LIB_PATH", str(tmp_path / "libcrgpu.so"))
    monkeypatch.setattr(N, "_lib", None)
    with pytest.raises(ImportError):
        N.lib()
