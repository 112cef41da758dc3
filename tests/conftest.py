import importlib.util
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


def load_package():
    """Import the product package (its directory name is not a Python identifier)."""
    name = "minipic_gb300"
    if name in sys.modules:
        return sys.modules[name]
    path = os.path.join(ROOT, "minipic-crossroads_gb300", "__init__.py")
    spec = importlib.util.spec_from_file_location(name, path)
    mod = importlib.util.module_from_spec(spec)
    sys.modules[name] = mod
    spec.loader.exec_module(mod)
    return mod


@pytest.fixture(scope="session")
def mpg():
    mod = load_package()
    mod.build()
    return mod


@pytest.fixture(scope="session")
def orc():
    from oracle import oracle as O
    O.build()
    return O
