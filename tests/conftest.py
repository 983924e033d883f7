import json
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (the parity tests proper)")
    config.addinivalue_line("markers", "slow: full-size workload")


def load_cases():
    with open(os.path.join(GOLDEN, "cases.json")) as f:
        return json.load(f)["cases"]


def case_id(c):
    return f"{c['graph']}-k{c['k']}-p{c['p']}-{'v2' if c['solver'].endswith('v2') else 'v1'}"


def matrix_path(c):
    return os.path.join(GOLDEN, c["matrix"])


@pytest.fixture(scope="session")
def gpu_ctx():
    from copsandrobbers_gb300.solver import Context

    ctx = Context(0)
    yield ctx
    ctx.close()
