import importlib.util
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG_DIR = os.path.join(ROOT, "test-regression_gb300")
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def _load_pkg():
    if "multifit_gb300" in sys.modules:
        return sys.modules["multifit_gb300"]
    spec = importlib.util.spec_from_file_location("multifit_gb300", os.path.join(PKG_DIR, "__init__.py"))
    mod = importlib.util.module_from_spec(spec)
    sys.modules["multifit_gb300"] = mod
    spec.loader.exec_module(mod)
    return mod


def _load_build():
    spec = importlib.util.spec_from_file_location("multifit_gb300_build", os.path.join(PKG_DIR, "build.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")
    config.addinivalue_line("markers", "slow: long-running CPU test")


@pytest.fixture(scope="session")
def mf():
    """The engine's Python host mirror; builds the library if it is missing."""
    _load_build().build()
    return _load_pkg()


@pytest.fixture(scope="session")
def oracle():
    import oracle as o

    o.lib()
    return o


@pytest.fixture(scope="session")
def cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


@pytest.fixture(scope="session")
def engine(mf, cuda):
    e = mf.Engine(0)
    yield e
    e.close()
