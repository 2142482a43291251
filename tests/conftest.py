import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)
HERE = os.path.dirname(os.path.abspath(__file__))
if HERE not in sys.path:
    sys.path.insert(0, HERE)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the product on the device)")
    config.addinivalue_line("markers", "slow: long-running")


@pytest.fixture(scope="session")
def gpu_op2():
    """pyop2_gb300.op2 with the native library built; fails loudly without it."""
    import torch
    if not torch.cuda.is_available():
        pytest.fail("GPU test collected on a machine without a CUDA device")
    from pyop2_gb300.csrc import build
    build.build()
    from pyop2_gb300 import op2, device
    device.require()
    return op2


@pytest.fixture(scope="session")
def oracle_op2():
    from oracle import op2
    return op2
