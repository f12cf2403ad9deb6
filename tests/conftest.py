import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the sm_103a library)")


@pytest.fixture(scope="session")
def gpu_lib():
    """Build (if needed) and load libpfemgpu.so.  GPU tests fail loudly if it cannot load."""
    from pfem_gb300 import api, build

    build.build()
    return api.load()


@pytest.fixture(scope="session")
def c1_mesh():
    from pfem_gb300 import mesh as M

    return M.dam_break_2d(0.05)


@pytest.fixture(scope="session")
def small3d_mesh():
    from pfem_gb300 import mesh as M

    return M.dam_break_3d(0.05, tank=(0.6, 0.3, 0.5), column=(0.2, 0.3, 0.3))


@pytest.fixture(scope="session")
def wc_small_mesh():
    from pfem_gb300 import mesh as M

    return M.dam_break_2d(0.02)
