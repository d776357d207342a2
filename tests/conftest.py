"""Shared fixtures.  GPU tests are marked ``gpu``; everything else runs on CPU."""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def hydro_lib():
    """The product library, built in-tree on first use."""
    from hydrofv_gb300 import build as B
    import hydrofv_gb300 as H
    if not os.path.exists(H.LIB_PATH):
        B.build()
    return H.library()


@pytest.fixture(scope="session")
def oracle_mod():
    """The CPU oracle (restatement; reference too when it was built)."""
    import oracle as O
    if not os.path.exists(os.path.join(O.BUILD, "liboracle.so")):
        O.build(with_reference=False)
    return O


@pytest.fixture(scope="session")
def gpu_available(hydro_lib):
    import hydrofv_gb300 as H
    if H.device_count() < 1:
        pytest.skip("no CUDA device visible")
    return True
