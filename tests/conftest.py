import gzip
import importlib
import json
import os
import sys
import tempfile

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
    path = os.path.join(GOLDEN, name)
    if name.endswith(".gz"):
        with gzip.open(path, "rt") as f:
            return json.load(f)
    with open(path) as f:
        return json.load(f)


def committed_cases():
    """Synthetic cases written here (the input file sits in tests/golden)."""
    return [c for c in golden_index() if "fixture" not in c]


def ieee_cases(max_buses=None):
    """The reference's own IEEE cases (input committed as ieee/*.cdf.gz)."""
    out = [c for c in golden_index() if "fixture" in c]
    if max_buses is not None:
        out = [c for c in out if ieee_buses(c) <= max_buses]
    return out


def ieee_buses(case):
    """Bus count of an IEEE case from its name: ieee<n> or ieee118x<k>."""
    name = case["cdf"][:-4]
    return 118 * int(name.split("x")[1]) if "x" in name else int(name[4:])


_UNPACKED = {}


def ieee_path(case):
    """Path of the decompressed input file of an IEEE case (once per session)."""
    fx = case["fixture"]
    if fx not in _UNPACKED:
        d = tempfile.mkdtemp(prefix="gbpf_ieee_")
        path = os.path.join(d, case["cdf"])
        with gzip.open(os.path.join(GOLDEN, fx), "rb") as f, open(path, "wb") as o:
            o.write(f.read())
        _UNPACKED[fx] = path
    return _UNPACKED[fx]


def case_path(case):
    return ieee_path(case) if "fixture" in case else os.path.join(GOLDEN, case["cdf"])
