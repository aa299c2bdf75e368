import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)
GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


def golden(name):
    import numpy as np
    return np.load(os.path.join(GOLDEN, name + ".npz"))


@pytest.fixture(scope="session")
def gpu_engine():
    from nrgplusplus_gb300 import api
    from nrgplusplus_gb300.build import build
    build(verbose=False)
    eng = api.Engine(api.PREC_FP64)
    yield eng
    eng.close()


@pytest.fixture(scope="session")
def mixed_engine():
    from nrgplusplus_gb300 import api
    from nrgplusplus_gb300.build import build
    build(verbose=False)
    eng = api.Engine(api.PREC_MIXED)
    yield eng
    eng.close()
