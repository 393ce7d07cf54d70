import json
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(ROOT / "tests"))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built libpcvl_gb300.so")
    config.addinivalue_line("markers", "slow: long-running case")


@pytest.fixture(scope="session")
def kats():
    return json.loads((ROOT / "tests" / "golden" / "reference_kats.json").read_text())


@pytest.fixture(scope="session")
def golden():
    return json.loads((ROOT / "tests" / "golden" / "golden_values.json").read_text())


@pytest.fixture(scope="session")
def oracle():
    from oracle import oracle as O
    O.build()
    return O


@pytest.fixture(scope="session")
def native():
    """The CUDA library, built in-tree if needed; fails (never skips) without a GPU."""
    import torch
    from perceval_gb300 import _build, _native
    if not _native.library_path().exists():
        _build.build()
    assert torch.cuda.is_available(), "GPU tests need CUDA"
    _native.load()
    return _native
