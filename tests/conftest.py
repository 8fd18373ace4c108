import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
PKG = ROOT / "gpe-matlab_gb300"
for p in (str(ROOT), str(PKG)):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a GB300 (sm_103) GPU and the built libgpe.so")
    config.addinivalue_line("markers", "slow: long-running case")


@pytest.fixture(scope="session")
def gpe():
    """The product package (loads libgpe.so; fails loudly if it is missing)."""
    import gpe_gb300

    if not gpe_gb300.device_available():
        pytest.fail("no sm_103 GPU visible: -m gpu tests need a GB300")
    return gpe_gb300
