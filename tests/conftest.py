import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (runs on the GB300 box)")
    # the engine library is built in-tree before any test imports the binding
    from multimodenonlinearoptics_gb300 import build_ext
    build_ext.build()


@pytest.fixture(scope="session")
def nlm():
    from multimodenonlinearoptics_gb300 import nonlinearmedium
    return nonlinearmedium


@pytest.fixture(scope="session")
def oracle():
    from oracle import nlm_oracle
    return nlm_oracle


@pytest.fixture(scope="session")
def golden():
    import numpy as np
    return np.load(os.path.join(ROOT, "tests", "golden", "oracle_golden.npz"))
