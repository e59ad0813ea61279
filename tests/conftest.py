import importlib.util
import json
import os
import sys

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(REPO, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); runs the CUDA library through its C-ABI")
    config.addinivalue_line("markers", "slow: longer CPU case")


def _load(name, path, pkg_dir=None):
    if name in sys.modules:
        return sys.modules[name]
    spec = importlib.util.spec_from_file_location(name, path,
                                                  submodule_search_locations=[pkg_dir] if pkg_dir else None)
    mod = importlib.util.module_from_spec(spec)
    sys.modules[name] = mod
    spec.loader.exec_module(mod)
    return mod


@pytest.fixture(scope="session")
def mh():
    pkg = os.path.join(REPO, "marinehydro.jl_gb300")
    return _load("marinehydro_gb300", os.path.join(pkg, "__init__.py"), pkg)


@pytest.fixture(scope="session")
def oracle():
    """The CPU oracle (test infrastructure only)."""
    return _load("oracle", os.path.join(REPO, "oracle", "oracle.py"))


@pytest.fixture(scope="session")
def kats():
    with open(os.path.join(GOLDEN, "reference_kats.json")) as f:
        return json.load(f)


@pytest.fixture(scope="session")
def ctx(mh):
    """A context on cuda:0.  GPU tests fail loudly when the library or the GPU is missing."""
    return mh.Context(0)
