import importlib
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden")
for p in (ROOT, os.path.join(ROOT, "oracle")):
    if p not in sys.path:
        sys.path.insert(0, p)

PKG = "magrathea-pathfinder_gb300"


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the sm_103a library)")


@pytest.fixture(scope="session")
def pkg():
    return importlib.import_module(PKG)


@pytest.fixture(scope="session")
def synth():
    return importlib.import_module(PKG + ".synth")


@pytest.fixture(scope="session")
def maps_mod():
    return importlib.import_module(PKG + ".maps")


def load_golden(name):
    return dict(np.load(os.path.join(GOLDEN, name + ".npz"), allow_pickle=False))


@pytest.fixture(scope="session", params=["uniform", "amr"])
def golden(request):
    g = load_golden(request.param)
    g["name"] = request.param
    return g


@pytest.fixture(scope="session")
def oracle_mod():
    import oracle
    oracle.build()
    return oracle


@pytest.fixture(scope="session")
def gpu_lib(pkg):
    """The native library on a real device; fails (does not skip) if absent."""
    build = importlib.import_module(PKG + ".build")
    build.build()
    L = pkg.library()
    assert L.mpf_device_count() > 0, "no CUDA device visible to libmpf_gb300.so"
    return L
