import os
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
sys.path.insert(0, str(ROOT / "dynearthsol-old_gb300"))
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(ROOT / "tests"))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")
    config.addinivalue_line("markers", "ref: needs the reference's own functions (oracle/_ref)")


@pytest.fixture(scope="session", autouse=True)
def built():
    from des_gb300.build import build
    build()
    from oracle import oracle
    oracle.build_oracle()
    return True


@pytest.fixture(scope="session")
def gpu():
    """Fails loudly (never skips) when the CUDA path cannot run."""
    import ctypes
    import des_gb300
    L = des_gb300.lib()
    return L
