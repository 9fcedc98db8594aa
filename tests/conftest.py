import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (ROOT, os.path.join(ROOT, "sfxc-1_gb300"), os.path.join(ROOT, "tests")):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300)")


@pytest.fixture(scope="session")
def oracle_exe():
    from oracle import build_oracle
    return build_oracle.build()


@pytest.fixture(scope="session")
def sfxc_lib():
    import build as sfxc_build
    sfxc_build.build()
    from sfxc_gpu import lib
    return lib.load()


@pytest.fixture(scope="session")
def gpu_node(sfxc_lib):
    from sfxc_gpu import correlator, lib
    node = correlator.CorrelatorNode(0, lib.X_FP32)
    yield node
    node.close()
