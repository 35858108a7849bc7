import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs on the GB300 host)")


@pytest.fixture(scope="session")
def orc():
    from oracle.oracle import Oracle
    return Oracle()


@pytest.fixture(scope="session")
def golden():
    import numpy as np
    d = os.path.join(ROOT, "tests", "golden")

    def load(name):
        return dict(np.load(os.path.join(d, name + ".npz")))
    return load


@pytest.fixture
def orc_pow(orc):
    """The oracle with Distance() spelled as the reference's powf calls, for
    bit-exact comparison with the reference's compiled outputs."""
    orc.lib.orc_set_pow_distance(1)
    yield orc
    orc.lib.orc_set_pow_distance(0)
