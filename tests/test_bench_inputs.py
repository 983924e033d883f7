"""The measured figures bench.py reads from committed files: the DRAM bytes of one solve step
and of one first-pass launch (ncu summaries), the copy peak, and the reference's own solver
timings.  They must parse and stay consistent with the algorithmic byte counts they sit beside
(no GPU)."""
import os
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
import bench  # noqa: E402

# the large solve's first pass: S table bytes + two marked planes + two flag planes
S = 2829056 * 256 * 2
ALG_FIRST_PASS = S + 2 * 2829056 * 8 * 4 + 2 * 2829056


def test_first_pass_traffic_is_close_to_its_algorithmic_bytes():
    t = bench.traffic_per_launch()
    assert t is not None
    assert 0.9 * ALG_FIRST_PASS < t <= 1.05 * ALG_FIRST_PASS


def test_solve_step_traffic_is_at_least_the_first_pass():
    solve, first = bench.solve_dram_bytes(), bench.traffic_per_launch()
    assert solve is not None and first is not None
    assert first <= solve < 1.2 * first   # the later passes stay mostly in L2


def test_peak_and_reference_timings_parse():
    peak, src = bench.measured_peak_hbm()
    assert peak > 1000.0 and src in ("measured", "fallback")
    ref = bench.reference_code_timings()
    assert ref is not None
    text = repr(ref)
    assert "k_cops_4" in text
