import os
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))

GOLDEN = ROOT / "tests" / "golden"


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (sm_103a) and the built libmillionsball")
    config.addinivalue_line("markers", "slow: full-size workloads")


@pytest.fixture(scope="session")
def built_lib():
    """Build (if stale) and load libmillionsball.so."""
    from bevy_millions_ball_gb300 import build as b
    from bevy_millions_ball_gb300 import _abi

    b.build()
    return _abi.load()


@pytest.fixture(scope="session")
def oracle_lib():
    import oracle

    return oracle.lib()


@pytest.fixture(scope="session")
def cuda():
    """torch with a visible CUDA device (device memory / streams for the stage API)."""
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch
