import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300)")


@pytest.fixture(scope="session")
def actx():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from actx_dgfem_suite_gb300.array_context import GB300DGArrayContext
    return GB300DGArrayContext("cuda:0")
