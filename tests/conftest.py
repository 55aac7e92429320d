import os
import sys

import numpy as np
import pytest

ROOT = os.path.abspath(os.path.join(os.path.dirname(__file__), ".."))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden", "reference_golden.npz")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def golden():
    return np.load(GOLDEN, allow_pickle=False)


@pytest.fixture(scope="session")
def orc():
    from oracle import Oracle, build

    build()
    return Oracle()


@pytest.fixture(scope="session")
def refl():
    """The reference's own compiled C++ (only where the reference sources exist)."""
    from oracle import RefLib, build_ref

    if not build_ref():
        pytest.skip("reference sources not present; golden fixtures cover this case")
    return RefLib()


@pytest.fixture(scope="session")
def lib():
    import radiosity_gb300 as R

    R.build()
    return R
