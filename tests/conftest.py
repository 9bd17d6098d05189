import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))

import __graft_entry__ as graft  # noqa: E402


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def oracle():
    return graft._load_module_file("ptf_oracle", ROOT / "oracle" / "ptf_oracle.py")


@pytest.fixture(scope="session")
def built_lib():
    """Path of libptf.so, building it when absent or stale."""
    b = graft._load_module_file("ptf_gb300_build", graft.PKG_DIR / "build.py")
    return b.build()


@pytest.fixture(scope="session")
def pkg(built_lib):
    return graft.load_package()


@pytest.fixture(scope="session")
def gpu(pkg):
    import torch
    if not torch.cuda.is_available():
        pytest.fail("GPU test run without a CUDA device")
    return pkg
