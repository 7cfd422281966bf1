import importlib
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (ROOT, os.path.join(ROOT, "oracle"), os.path.dirname(os.path.abspath(__file__))):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs on a GB300)")


def pkg(name=""):
    return importlib.import_module("cuacd-web_gb300" + (("." + name) if name else ""))


@pytest.fixture(scope="session")
def oracle():
    import harness

    harness.lib()
    return harness
