"""Shared pytest configuration.

``-m gpu`` tests need a CUDA device and the in-tree library; everything else
runs on the CPU.  The library is built (or found up to date) once per session.
"""

import os
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))

# the serving tests run several streams at once: the CUDA context (created
# later, by the first GPU test) gets as many hardware work queues
os.environ.setdefault("CUDA_DEVICE_MAX_CONNECTIONS", "32")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300, sm_103a)")


@pytest.fixture(scope="session")
def native_lib():
    from probit_gb300 import build, _native

    build.build()
    return _native.load()


@pytest.fixture(scope="session")
def cuda_device(native_lib):
    import torch

    if not torch.cuda.is_available():
        pytest.fail("gpu test run without a CUDA device")
    return torch.device("cuda", 0)
