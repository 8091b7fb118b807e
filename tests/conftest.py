import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "hydrangea-compiler_gb300")
for p in (ROOT, PKG):
    if p not in sys.path:
        sys.path.insert(0, p)

# keep the autotuner's on-disk cache of this test session out of $HOME
if "HYD_CUDA_TUNE_CACHE" not in os.environ:
    import tempfile
    os.environ["HYD_CUDA_TUNE_CACHE"] = os.path.join(tempfile.mkdtemp(prefix="hyd_tune_"), "tune.tsv")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


def _has_gpu():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


def pytest_collection_modifyitems(config, items):
    if _has_gpu():
        return
    skip = pytest.mark.skip(reason="no CUDA GPU in this environment")
    for item in items:
        if "gpu" in item.keywords:
            item.add_marker(skip)


@pytest.fixture(scope="session")
def hc():
    import hyd_cuda
    hyd_cuda.lib()
    return hyd_cuda


@pytest.fixture(scope="session")
def orc():
    from oracle import oracle as O
    O.lib()
    return O


@pytest.fixture(scope="session")
def dev(hc):
    import torch
    d = torch.device("cuda:0")
    torch.cuda.set_device(d)
    hc.check(hc.lib().hyd_cuda_init())
    return d
