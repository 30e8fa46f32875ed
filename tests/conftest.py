import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "tests"))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def vko():
    import oracle_bind

    return oracle_bind


@pytest.fixture(scope="session")
def gb():
    """The GPU library, built for sm_103a (raises if it cannot be built or loaded)."""
    import vkvg_gb300

    vkvg_gb300._build.build()
    vkvg_gb300.lib()
    return vkvg_gb300
