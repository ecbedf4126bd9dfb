import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))

# z2d source tree with the golden PNGs; only present where the reference is
# mounted (golden checks of the oracle skip elsewhere).
Z2D_TREE = os.environ.get("Z2D_REFERENCE_TREE", "/root/reference")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (run with -m gpu)")


@pytest.fixture(scope="session")
def oracle():
    from oracle import Oracle
    return Oracle()


@pytest.fixture(scope="session")
def golden_dir():
    d = os.path.join(Z2D_TREE, "spec", "files")
    if not os.path.isdir(d):
        pytest.skip("z2d spec goldens not present on this machine")
    return d
