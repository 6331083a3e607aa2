"""Shared fixtures.  GPU tests carry @pytest.mark.gpu and call the CUDA path through the
C ABI; everything else runs on the CPU (oracle, host logic, ABI exports)."""
import importlib
import os
import sys

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = "dynamic-occupancy-grid-map_gb300"
for p in (REPO, os.path.join(REPO, "oracle"), os.path.join(REPO, "tests")):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the sm_103a kernels)")


def _build():
    spec = importlib.util.spec_from_file_location("dogm_gb300_build", os.path.join(REPO, PKG, "build.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


@pytest.fixture(scope="session")
def oracle():
    _build().build_oracle()
    import pyoracle
    pyoracle.load()
    return pyoracle


@pytest.fixture(scope="session")
def dogm():
    _build().build_cuda()
    mod = importlib.import_module(PKG)
    mod.load()
    return mod


@pytest.fixture(scope="session")
def scene():
    return importlib.import_module(PKG + ".scene")


@pytest.fixture(scope="session")
def pyref():
    """The reference's own CUDA build (oracle/pyref.py); skips where its cubins are absent."""
    _build().build_ref_harness()
    import pyref as mod
    why = mod.missing()
    if why:
        pytest.skip(why)
    mod.load()
    return mod
