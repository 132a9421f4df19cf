import os
import sys

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG_DIR = os.path.join(REPO, "avocado-sandwich_gb300")
for p in (PKG_DIR, REPO):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def oracle_mod():
    import oracle
    oracle.build()
    return oracle


@pytest.fixture(scope="session")
def avs_mod():
    """The CUDA library binding; built in-tree if needed.  No fallback."""
    import avs
    from avs import build as avs_build
    if not os.path.exists(avs.library_path()):
        avs_build.build()
    avs.lib()
    return avs
