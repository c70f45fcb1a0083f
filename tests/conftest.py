"""Shared pytest configuration: the `gpu` marker and build-on-demand of the
in-tree library and the oracle."""
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")
    config.addinivalue_line("markers", "slow: long-running case")


@pytest.fixture(scope="session")
def gblib():
    """The gbchol shared library (built in-tree if missing)."""
    from cholespy_gb300 import _build, _ffi
    _build.build()
    return _ffi.lib()


@pytest.fixture(scope="session")
def oracle_lib():
    import oracle
    oracle.build()
    return oracle


@pytest.fixture(scope="session")
def cuda():
    import torch
    if not torch.cuda.is_available():
        pytest.fail("CUDA device required for gpu-marked tests")
    from cholespy_gb300 import _build
    _build.build()
    return torch
