import importlib.util
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a GB300 and the built CUDA engine")
    config.addinivalue_line("markers", "slow: larger CPU-side cases")


def load_engine():
    """Import the engine package (directory ``qaintensor.jl_gb300``) as ``qaintensor_gb300``."""
    if "qaintensor_gb300" in sys.modules:
        return sys.modules["qaintensor_gb300"]
    pkg_dir = os.path.join(ROOT, "qaintensor.jl_gb300")
    spec = importlib.util.spec_from_file_location(
        "qaintensor_gb300", os.path.join(pkg_dir, "__init__.py"), submodule_search_locations=[pkg_dir])
    mod = importlib.util.module_from_spec(spec)
    sys.modules["qaintensor_gb300"] = mod
    spec.loader.exec_module(mod)
    return mod


@pytest.fixture(scope="session")
def engine():
    return load_engine()


@pytest.fixture(scope="session")
def gpu_handle_factory(engine):
    """Creates engine handles on cuda:0; fails loudly when the library is missing."""
    handles = []

    def make(**cfg):
        h = engine.Engine(**cfg)
        handles.append(h)
        return h

    yield make
    for h in handles:
        h.close()
