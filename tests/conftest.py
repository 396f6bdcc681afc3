import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "tests"))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def oracle():
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import pyoracle

    pyoracle.build(with_ref=False)
    return pyoracle


@pytest.fixture(scope="session")
def native():
    from solidfmm_gb300 import build

    build.build()
    import solidfmm_gb300

    return solidfmm_gb300
