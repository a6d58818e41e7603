import sys
from pathlib import Path

import pytest

REPO = Path(__file__).resolve().parent.parent
# The oracle binding (oracle/oracle.py) must win over the oracle/ directory.
for p in (str(REPO), str(REPO / "stochastic-parker_gb300"), str(REPO / "oracle")):
    if p in sys.path:
        sys.path.remove(p)
    sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")
    config.addinivalue_line("markers", "slow: long-running statistical check")


def _cuda_available() -> bool:
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


def pytest_collection_modifyitems(config, items):
    if _cuda_available():
        return
    skip = pytest.mark.skip(reason="no CUDA device")
    for item in items:
        if "gpu" in item.keywords:
            item.add_marker(skip)


@pytest.fixture(scope="session")
def engine_lib():
    from gpat import build, _abi
    build.build()
    return _abi.load()


@pytest.fixture(scope="session")
def orc():
    import oracle
    oracle.load()
    return oracle
