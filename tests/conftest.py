import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)
GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and libafem_gb300.so")


@pytest.fixture(scope="session")
def cuda_ctx():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from arcanefem_gb300 import fem
    ctx = fem.Context()
    yield ctx
    ctx.close()
