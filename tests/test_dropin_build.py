"""The second integration route: the reference's own driver (app/main.cpp) and lib/ compiled with
the GPU solver translation unit in place of one of its solvers (-DALGORITHM_INCLUDE), for both
rule sets.  Compilation only (runs need a GPU; tests/test_dropin_gpu.py runs the drop-in
executables).  Needs the reference tree (CR_REFERENCE_ROOT); skipped where it is absent."""
import glob
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REF = os.environ.get("CR_REFERENCE_ROOT", "/root/reference")
LIB = os.path.join(ROOT, "copsandrobbers_gb300")


@pytest.mark.skipif(not os.path.exists(os.path.join(REF, "app", "main.cpp")), reason="reference tree absent")
@pytest.mark.skipif(not os.path.exists(os.path.join(LIB, "libcrgpu.so")), reason="libcrgpu.so not built")
@pytest.mark.parametrize("rules", [1, 2])
def test_reference_driver_builds_with_gpu_solver(tmp_path, rules):
    cxx = shutil.which("g++")
    if not cxx:
        pytest.skip("g++ absent")
    tu = os.path.join(LIB, "csrc", "k_cops_gpu.cpp")
    out = tmp_path / f"k_cops_gpu_v{rules}.exe"
    cmd = [cxx, "-std=c++17", "-include", "cstddef", "-O1", "-I", os.path.join(REF, "lib", "include"),
           "-I", os.path.join(ROOT, "include"), f'-DALGORITHM_INCLUDE="{tu}"', f"-DCR_GPU_RULES={rules}",
           os.path.join(REF, "app", "main.cpp"), *sorted(glob.glob(os.path.join(REF, "lib", "src", "*.cpp"))),
           "-L", LIB, "-lcrgpu", f"-Wl,-rpath,{LIB}", "-o", str(out)]
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-3000:]
    assert out.exists()
