"""Shared fixtures.  `gpu` marks tests that need a CUDA device; everything
else runs on CPU.  The oracle (oracle/) is the checker in these tests."""
import os
import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parent.parent
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs on the GB300)")


@pytest.fixture(scope="session")
def built():
    """Build the product library and the oracle once per session."""
    from skwarka_gb300 import build as pbuild
    from oracle import build as obuild
    pbuild.build()
    obuild.build_oracle()
    return True


@pytest.fixture(scope="session")
def oracle(built):
    from oracle.api import Oracle
    return Oracle()


@pytest.fixture(scope="session")
def reference(built):
    """The reference's own code, or skip where it is not built."""
    from oracle import build_ref
    from oracle.api import Reference
    if not Reference.available():
        try:
            build_ref.build()
        except Exception as e:  # pragma: no cover - depends on the machine
            pytest.skip(f"reference build unavailable: {e}")
    if not Reference.available():
        pytest.skip("reference sources not available on this machine")
    return Reference()


def cuda_ok() -> bool:
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.fixture(scope="session")
def gpu(built):
    if not cuda_ok():
        pytest.skip("no CUDA device")
    import torch
    torch.cuda.init()
    return torch.device("cuda:0")
