import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKGDIR = os.path.join(ROOT, "3d-bi-anisotropic-phc_gb300")
for p in (PKGDIR, ROOT):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def fame_lib():
    """The in-tree CUDA library, built on first use if absent."""
    import fame
    from fame.build import build_library

    if not os.path.exists(fame.lib_path()):
        build_library()
    return fame.load()


@pytest.fixture(scope="session")
def cuda():
    import torch

    if not torch.cuda.is_available():
        pytest.fail("GPU test without a CUDA device")
    torch.cuda.set_device(0)
    return torch.device("cuda:0")
