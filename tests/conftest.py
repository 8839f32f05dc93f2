import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

import __graft_entry__ as _entry  # noqa: E402


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def tg():
    """The product package (host mirror + CUDA library binding)."""
    return _entry.load_package()


@pytest.fixture(scope="session")
def orc():
    """The CPU oracle (checker)."""
    mod = _entry.load_oracle()
    odir = os.path.join(ROOT, "oracle")
    if odir not in sys.path:
        sys.path.insert(0, odir)
    mod.build()
    return mod


@pytest.fixture(scope="session")
def gpu_lib(tg):
    """Built and loaded CUDA library (GPU tests only)."""
    import importlib
    importlib.import_module("trixiatmo_gb300.build").build()
    return tg._lib.load(build_if_missing=False)
