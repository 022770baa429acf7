import os
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
GOLDEN = ROOT / "tests" / "golden"
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); runs the CUDA path through the C ABI")


@pytest.fixture(scope="session")
def golden() -> Path:
    return GOLDEN


@pytest.fixture(scope="session")
def oracle():
    from oracle import oracle as O
    O.build()
    return O


@pytest.fixture(scope="session")
def native_built():
    from trinityrnaseq_gb300.build import build
    return build()


@pytest.fixture(scope="session")
def ctx(native_built):
    from trinityrnaseq_gb300 import Context
    c = Context(int(os.environ.get("TK_DEVICE", "0")))
    yield c
    c.close()
