import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (ROOT, os.path.join(ROOT, "oracle"), os.path.join(ROOT, "tests")):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def oracle():
    """The C restatement (built on first use with gcc)."""
    import oracle_py

    oracle_py.build_oracle()
    return oracle_py


@pytest.fixture(scope="session")
def mhdlib():
    """The product library (built on first use with nvcc)."""
    from ppkmhd_gb300 import build

    build.build()
    import ppkmhd_gb300

    return ppkmhd_gb300
