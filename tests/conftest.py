import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)
GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); run with -m gpu")


@pytest.fixture(scope="session")
def built():
    """Builds the native library, CLI and oracle in-tree once per session."""
    from gpuothello2_gb300 import build

    build.build_library()
    build.build_oracle()
    build.build_host()
    return build


@pytest.fixture(scope="session")
def oracle(built):
    from tests.oracle_lib import Oracle

    return Oracle(built.ORACLE_LIB)


@pytest.fixture(scope="session")
def gpu(built):
    """The native library on a GPU; skips the test when no GPU is visible."""
    import gpuothello2_gb300 as g

    try:
        g.device_info()
    except Exception as e:  # no device in this process
        pytest.skip("no CUDA device: %s" % e)
    return g
