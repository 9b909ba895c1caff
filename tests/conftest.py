import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def built():
    """The product library and the oracle library, built in-tree if missing."""
    from emc_gb300 import _lib
    from oracle import build as OB
    if not _lib.LIB_PATH.exists():
        from emc_gb300 import build as B
        B.build()
    OB.build()
    return _lib.load()


@pytest.fixture(scope="session")
def cuda(built):
    import torch
    assert torch.cuda.is_available(), "GPU tests need a CUDA device"
    return torch.device("cuda:0")


@pytest.fixture(scope="session")
def ctx(cuda):
    import emc_gb300 as E
    c = E.Context(0)
    yield c
    c.close()
