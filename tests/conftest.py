import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))

# z2d source tree with the golden PNGs: $Z2D_REFERENCE_TREE, or a checkout
# named "reference" beside this repository.  Golden checks of the oracle skip
# where neither exists.
Z2D_TREE = os.environ.get("Z2D_REFERENCE_TREE", os.path.join(os.path.dirname(ROOT), "reference"))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (run with -m gpu)")
    # the rasteriser's autotuner caches its choices in this session's own file
    if "Z2D_TUNE_FILE" not in os.environ:
        import tempfile
        os.environ["Z2D_TUNE_FILE"] = os.path.join(tempfile.mkdtemp(prefix="z2d_tune_"), "raster_tune.json")


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
