import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); runs the CUDA path")


@pytest.fixture(scope="session")
def oracle():
    import pyoracle
    pyoracle.build(ref=True)
    return pyoracle


@pytest.fixture(scope="session")
def native():
    from owlexastitcher_gb300 import build
    build.build_all()
    return build


def dataset(config, **kw):
    from owlexastitcher_gb300 import datagen
    return datagen.Dataset(config, **kw)
