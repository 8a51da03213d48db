import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def oracle():
    from oracle import pyoracle
    pyoracle.build()
    return pyoracle


@pytest.fixture(scope="session")
def stslib():
    import ceda_demonstrations_gb300 as sts
    sts.lib()
    return sts


@pytest.fixture(scope="session")
def ctx(stslib):
    if stslib.lib().STS_DeviceCount() < 1:
        pytest.fail("no CUDA device visible: GPU tests need a GB300")
    return stslib.Context(0)
