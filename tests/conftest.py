"""Shared fixtures. GPU tests are marked ``gpu``; everything else runs on CPU."""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parent.parent
GOLDEN = ROOT / "tests" / "golden"
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the CUDA library)")


@pytest.fixture(scope="session")
def port():
    from oracle import oracle as O
    return O.port()


@pytest.fixture(scope="session")
def ref():
    from oracle import oracle as O
    try:
        O.build_ref()
    except Exception:
        pass
    r = O.ref()
    if r is None:
        pytest.skip("reference sources not mounted here (pinned by tests/golden instead)")
    return r


@pytest.fixture(scope="session")
def cuda_lib():
    from bonxai_gb300 import build as B
    B.build()
    import bonxai_gb300 as bx
    return bx.load_library()


@pytest.fixture(scope="session")
def gpu(cuda_lib):
    import torch
    assert torch.cuda.is_available(), "GPU tests need a CUDA device"
    torch.cuda.set_device(0)
    import bonxai_gb300 as bx
    return bx


def golden(name):
    return np.load(GOLDEN / name)
