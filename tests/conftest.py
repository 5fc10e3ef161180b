import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300 / sm_103a)")


@pytest.fixture(scope="session")
def oracle():
    from oracle.nxo import Oracle, build
    build(ref=False)
    return Oracle()


@pytest.fixture(scope="session")
def reference():
    """The reference compiled from its own sources (skips where its tree is absent)."""
    from oracle import nxo
    if not nxo.reference_available():
        pytest.skip("reference library not built and NXM_REFERENCE_TREE not set")
    nxo.build(ref=True)
    return nxo.Reference()


@pytest.fixture(scope="session")
def c1_compat():
    """Config-1 shaped system made well-behaved under the reference's derived box."""
    from nexusmd_gb300 import synthetic as sy
    return sy.compat_system(sy.config_system(1))


@pytest.fixture(scope="session")
def small_compat():
    """A ~900-atom chain + water system for quick multi-step checks."""
    from nexusmd_gb300 import synthetic as sy
    return sy.compat_system(sy.make_system(1, 20, 240, 2.4, seed=77, grid=(24, 24, 24)))
