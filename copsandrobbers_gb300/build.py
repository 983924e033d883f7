"""Builds the native parts of the package in-tree.

* ``libcrgpu.so``  - the CUDA kernels and the C ABI of ``include/crgpu.h`` (sm_103a only).
* ``bin/k_cops_gpu``, ``bin/k_cops_gpu_v2`` - the drop-in solver executables (v1 / v2 rules): the six-phase solver translation unit
  ``csrc/k_cops_gpu.cpp`` behind a driver with the reference's argv and stdout contract.

Each translation unit is compiled in parallel with ``nvcc -gencode arch=compute_103a,code=sm_103a``;
objects are reused while they are newer than their sources and headers.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OBJ = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libcrgpu.so")
BIN = os.path.join(HERE, "bin")
EXE = os.path.join(BIN, "k_cops_gpu")

CU_SOURCES = ["crgpu_api.cu", "crgpu_v1.cu", "crgpu_v2.cu", "crgpu_tables.cu", "crgpu_batch.cu",
              "crgpu_noalloc.cu", "crgpu_server.cu"]
HEADERS = ["crgpu_internal.cuh", "crgpu_v1_body.cuh", "crgpu_ctx.h", "crgpu_v2.h",
           os.path.join("..", "..", "include", "crgpu.h")]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libcrgpu.so")


def _stale(target: str, deps: list[str]) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.exists(d) and os.path.getmtime(d) > t for d in deps)


def _compile(src: str) -> str:
    obj = os.path.join(OBJ, os.path.splitext(src)[0] + ".o")
    deps = [os.path.join(CSRC, src)] + [os.path.join(CSRC, h) for h in HEADERS]
    missing = [d for d in deps if not os.path.exists(d)]
    if missing:
        raise RuntimeError(f"build dependencies missing: {missing}")
    if _stale(obj, deps):
        cmd = [nvcc(), *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
               "-I", os.path.join(ROOT, "include"), "-c", os.path.join(CSRC, src), "-o", obj]
        subprocess.run(cmd, check=True)
    return obj


def build(verbose: bool = False) -> str:
    os.makedirs(OBJ, exist_ok=True)
    os.makedirs(BIN, exist_ok=True)
    srcs = [s for s in CU_SOURCES if os.path.exists(os.path.join(CSRC, s))]
    with cf.ThreadPoolExecutor(max_workers=len(srcs)) as ex:
        objs = list(ex.map(_compile, srcs))
    if _stale(LIB, objs):
        subprocess.run([nvcc(), *ARCH, "-shared", "-o", LIB, *objs, "-lcudart"], check=True)
    solver_srcs = [os.path.join(CSRC, "k_cops_gpu.cpp"), os.path.join(CSRC, "k_cops_gpu_main.cpp")]
    for exe, rules in ((EXE, 1), (EXE + "_v2", 2)):
        if _stale(exe, solver_srcs + [LIB, os.path.join(ROOT, "include", "crgpu.h")]):
            cxx = shutil.which("g++") or "g++"
            subprocess.run([cxx, "-std=c++17", "-O2", "-Wall", "-I", os.path.join(ROOT, "include"),
                            "-I", CSRC, '-DCR_SOLVER_TU="k_cops_gpu.cpp"', f"-DCR_GPU_RULES={rules}",
                            solver_srcs[1], "-o", exe, "-L", HERE, "-lcrgpu",
                            f"-Wl,-rpath,{HERE}"], check=True)
    if verbose:
        print(f"built {LIB}")
    return LIB


if __name__ == "__main__":
    build(verbose=True)
    sys.exit(0)
