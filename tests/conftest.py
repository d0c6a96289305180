import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
for p in (ROOT, ROOT / "tests"):
    if str(p) not in sys.path:
        sys.path.insert(0, str(p))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (sm_103a) and the built library")
    config.addinivalue_line("markers", "slow: long-running parity run")


@pytest.fixture(scope="session")
def oracle_lib():
    import oracle

    return oracle.lib()
