"""The drop-in executables (the six-phase solver translation unit behind a driver with the
reference's argv) print the reference's stdout lines and write its cache file byte for byte."""
import hashlib
import os
import shutil
import subprocess

import pytest

from conftest import case_id, load_cases, matrix_path
from oracle import oracle as O

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
BIN = os.path.join(ROOT, "copsandrobbers_gb300", "bin")
CASES = [c for c in load_cases() if (c["graph"] in ("peterson", "grid9", "dodecahedron", "planar8")
         and c["k"] <= 2 and c["p"] <= 2) or (c["graph"] == "peterson" and c["k"] == 3)]


def run(exe, workdir, graph_file, k, p):
    return subprocess.run([os.path.join(BIN, exe), graph_file, str(k), str(p)], cwd=workdir,
                          capture_output=True, text=True, timeout=120)


@pytest.mark.parametrize("case", CASES, ids=case_id)
def test_dropin_stdout_and_table_file(case, tmp_path):
    exe = "k_cops_gpu_v2" if case["solver"].endswith("v2") else "k_cops_gpu"
    src = matrix_path(case)
    shutil.copyfile(src, tmp_path / os.path.basename(src))
    for attempt in range(2):  # the second run finds the cache file (a hit solves identically)
        proc = run(exe, tmp_path, os.path.basename(src), case["k"], case["p"])
        assert proc.returncode == 0, proc.stderr
        out = proc.stdout
        assert "[FAILED STEP]" not in out
        assert ("Loaded AuxGraph from cache!" in out) == (attempt == 1)
        assert [int(b) for _, b in O.RE_PASS.findall(out)] == case["pass_counts"]
        assert int(O.RE_CAPS.search(out).group(1)) == case["base_captures"]
        assert O.RE_RESULT.search(out).group(1) == case["result"]
        if case["result"] == "WIN":
            assert O.RE_POS.search(out).group(1) == case["positions"]
            assert int(O.RE_CAPTURE.search(out).group(1)) == case["capture_plies"]
        assert O.RE_MAINLOOP.search(out) is not None                  # timing report line
        assert "Total Footprint" in out and "Saving filled AuxGraph to cache... Success!" in out
        table = tmp_path / "cache" / case["table_file"]
        assert table.exists(), sorted(os.listdir(tmp_path / "cache"))
        assert hashlib.sha256(table.read_bytes()).hexdigest() == case["sha_file"]


def test_dropin_usage_and_bad_file(tmp_path):
    proc = subprocess.run([os.path.join(BIN, "k_cops_gpu")], capture_output=True, text=True)
    assert proc.returncode == 1 and "Usage:" in proc.stdout
    (tmp_path / "empty.txt").write_text("")
    proc = run("k_cops_gpu", tmp_path, "empty.txt", 2, 1)
    assert proc.returncode == 0
    assert "[FAILED STEP]: 'Load Graph File' was unsuccessful!" in proc.stdout
