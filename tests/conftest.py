import os
import sys

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (os.path.join(REPO, "ct-xafs_analysis_gb300"), os.path.join(REPO, "oracle"), REPO):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (sm_103, GB300)")


@pytest.fixture(scope="session")
def oracle_lib():
    import oracle
    oracle.build()
    return oracle


@pytest.fixture(scope="session")
def xct_lib():
    """libxct.so, built in-tree if missing (nvcc cross-compiles without a GPU)."""
    import xct
    from xct import build
    if not os.path.exists(xct.LIB_PATH):
        build.build_lib()
    return xct.load()


@pytest.fixture(scope="session")
def gpu_ctx(xct_lib):
    import torch
    if not torch.cuda.is_available():
        pytest.fail("GPU test run without a CUDA device")
    import xct
    ctx = xct.Context(0)
    yield ctx
    ctx.close()
