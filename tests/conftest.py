import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the sm_103a kernels)")


@pytest.fixture(scope="session")
def orc():
    from oracle.oracle import Oracle
    return Oracle()


@pytest.fixture(scope="session")
def golden():
    return dict(np.load(os.path.join(ROOT, "tests", "golden", "ref_golden.npz")))


@pytest.fixture(scope="session")
def ginputs():
    from tests.golden.make_golden import golden_inputs
    return golden_inputs()


@pytest.fixture(scope="session")
def ctx():
    from mambatracer_gb300 import api
    c = api.Context(0)
    yield c
    c.close()
