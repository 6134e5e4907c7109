import json
import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
GOLDEN = ROOT / "tests" / "golden"
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); runs the engine through its C ABI")


def golden(name):
    return json.loads((GOLDEN / name).read_text())


def unhex(xs):
    return np.array([float.fromhex(x) for x in xs])


@pytest.fixture(scope="session")
def engine():
    from hestonexotics_gb300 import Engine
    e = Engine(0)
    yield e
    e.close()


@pytest.fixture(scope="session")
def oracle():
    from oracle import oracle as O
    O.build()
    return O
