import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the sm_103a kernels)")


@pytest.fixture(scope="session")
def oracle():
    import oracle_lib
    return oracle_lib


@pytest.fixture(scope="session")
def cuda_lib():
    """The built nt2cuda library; builds it when missing."""
    import nt2_gb300.build as b
    b.build()
    import nt2_gb300
    return nt2_gb300.lib()


@pytest.fixture(scope="session")
def gpu(cuda_lib):
    import torch
    if not torch.cuda.is_available():
        pytest.fail("GPU test collected without a CUDA device")
    import nt2_gb300.api as api
    api.init(0)
    return api
