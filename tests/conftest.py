import os
import sys
from pathlib import Path

import pytest

# every BVH built during the tests is checked on the host for structure
os.environ.setdefault("PT_VALIDATE_BVH", "1")
# the two-pass extend (step budget, parked rays resumed) runs on waves of
# every size here, not only on the large waves it is used for by default, so
# the parity tests cover it; the one-pass form is covered by the
# execution-variant tests (which set their own environment)
os.environ.setdefault("PT_EXTEND_BUDGET_MIN_LOG2", "0")

ROOT = Path(__file__).resolve().parent.parent
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); runs the CUDA path through the C ABI")


@pytest.fixture(scope="session", autouse=True)
def native_build():
    """Make sure the oracle and the product library are built (fast no-op when up to date)."""
    import oracle
    from pt_gb300 import build as native
    oracle.build()
    native.build()
    yield


@pytest.fixture(scope="session")
def has_gpu():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False
