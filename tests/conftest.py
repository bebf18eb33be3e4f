import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); runs the native CUDA path")


@pytest.fixture(scope="session")
def built():
    """Build the native library, the generator and the oracle once."""
    import __graft_entry__
    __graft_entry__.build()
    return True


@pytest.fixture()
def shm_dir(tmp_path_factory):
    base = "/dev/shm" if os.path.isdir("/dev/shm") else None
    import tempfile
    d = tempfile.mkdtemp(prefix="gfs_t_", dir=base)
    yield d
    import shutil
    shutil.rmtree(d, ignore_errors=True)
