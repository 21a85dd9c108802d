import json
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "starformationhistories.jl_gb300")
for p in (os.path.join(ROOT, "oracle"), PKG, ROOT):
    if p not in sys.path:
        sys.path.insert(0, p)

GOLDEN_DIR = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a GB300 GPU (calls the CUDA library)")


@pytest.fixture(scope="session")
def O():
    """The FP64 CPU oracle (test infrastructure)."""
    import oracle as _o
    _o.build()
    return _o


@pytest.fixture(scope="session")
def kats():
    with open(os.path.join(GOLDEN_DIR, "reference_kats.json")) as f:
        return json.load(f)


@pytest.fixture(scope="session")
def sfh():
    """The product package; loading fails loudly when libsfhgpu.so is unusable."""
    import sfhgpu
    sfhgpu.load()
    return sfhgpu


@pytest.fixture(scope="session")
def ctx(sfh):
    return sfh.default_context()
