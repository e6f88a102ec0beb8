import json
import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parent.parent
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(ROOT / "oracle"))
GOLDEN = ROOT / "tests" / "golden"


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built libvjgb")
    config.addinivalue_line("markers", "slow: takes more than a few seconds on the CPU")


@pytest.fixture(scope="session")
def golden():
    return json.loads((GOLDEN / "golden.json").read_text())


@pytest.fixture(scope="session")
def gin():
    return dict(np.load(GOLDEN / "inputs.npz"))


@pytest.fixture(scope="session")
def oracle():
    import oracle as O
    O.lib()
    return O


@pytest.fixture(scope="session")
def vj():
    import cs677s26_gb300 as V
    V.load()
    return V


@pytest.fixture(scope="session")
def basic_pool(oracle):
    return oracle.feature_pool(0)


@pytest.fixture(scope="session")
def cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


def f32(bits: int) -> float:
    return float(np.uint32(bits).view(np.float32))


def f32bits(x) -> int:
    return int(np.array([x], dtype=np.float32).view(np.uint32)[0])
