import importlib.util
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs on the GB300 box)")
    config.addinivalue_line("markers", "slow: long CPU replay; still part of the default suite")


def load_package():
    """The product package lives in the directory `inspire-rs_gb300/`; import it under
    the module name `inspire_gb300`."""
    if "inspire_gb300" in sys.modules:
        return sys.modules["inspire_gb300"]
    pkg_dir = os.path.join(ROOT, "inspire-rs_gb300")
    spec = importlib.util.spec_from_file_location(
        "inspire_gb300", os.path.join(pkg_dir, "__init__.py"), submodule_search_locations=[pkg_dir])
    mod = importlib.util.module_from_spec(spec)
    sys.modules["inspire_gb300"] = mod
    spec.loader.exec_module(mod)
    return mod


@pytest.fixture(scope="session")
def oracle():
    from oracle import oracle as O
    O.build()
    return O


@pytest.fixture(scope="session")
def recorded_lines():
    with open(os.path.join(ROOT, "tests", "golden", "seat_kat_lines.txt")) as f:
        return f.read().splitlines()
