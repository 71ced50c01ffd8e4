"""Test configuration: the `gpu` marker, import paths and shared builders."""
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
for p in (ROOT / "casm-hella_gb300", ROOT / "oracle", ROOT / "tests"):
    if str(p) not in sys.path:
        sys.path.insert(0, str(p))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs on the GB300 box)")


@pytest.fixture(scope="session")
def oracle():
    import oracle as o
    o.build()
    return o


@pytest.fixture(scope="session")
def hella():
    """The product library's binding; builds the library first (sm_103a)."""
    import build as b
    b.build()
    import hella_gb300
    hella_gb300.lib()
    return hella_gb300
