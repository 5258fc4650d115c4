import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (ROOT, os.path.join(ROOT, "wfa2-lib_gb300"), os.path.join(ROOT, "tests")):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def oracle_mod():
    from oracle import oracle as O
    O.build(ref=False)
    return O


@pytest.fixture(scope="session")
def wfa():
    import wfa2gpu as W
    W.build()
    return W


@pytest.fixture(scope="session")
def gpu_available(wfa):
    if wfa.lib().wfa2gpu_device() < 0:
        pytest.fail("no CUDA device visible: GPU tests must run on a GPU host")
    return True
