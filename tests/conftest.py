import os
import sys

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, REPO)
sys.path.insert(0, os.path.join(REPO, "oracle"))
sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and libnyles_gb300.so")


@pytest.fixture(autouse=True)
def _unfreeze_parameters():
    from nyles_gb300 import parameters
    parameters.InextensibleDict.unfreeze()
    yield
    parameters.InextensibleDict.unfreeze()
