"""Test configuration: the `gpu` marker, repo-root imports, and one-time builds."""
import os
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (run with -m gpu)")


@pytest.fixture(scope="session")
def built_lib():
    from ncarray_gb300 import build
    build.build()
    from ncarray_gb300 import _lib
    return _lib.lib()


@pytest.fixture(scope="session")
def orc():
    import oracle
    oracle.build(with_ref=None)
    oracle.lib()
    return oracle


@pytest.fixture(scope="session")
def cuda(built_lib):
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    torch.cuda.set_device(0)
    return torch
