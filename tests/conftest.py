import importlib
import json
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden")
REFERENCE_GPU = "/root/reference/GPU"
PKG = "experience-of-using-gpu-in-power-flow-computation_gb300"

sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the sm_103a kernels)")


@pytest.fixture(scope="session")
def gb():
    return importlib.import_module(PKG)


@pytest.fixture(scope="session")
def oracle():
    import oracle as o

    o.lib()
    return o


def golden_index():
    with open(os.path.join(GOLDEN, "index.json")) as f:
        return json.load(f)


def load_golden(name):
    with open(os.path.join(GOLDEN, name)) as f:
        return json.load(f)


def committed_cases():
    return [c for c in golden_index() if os.path.exists(os.path.join(GOLDEN, c["cdf"]))]


def ieee_cases():
    return [c for c in golden_index() if not os.path.exists(os.path.join(GOLDEN, c["cdf"]))]
