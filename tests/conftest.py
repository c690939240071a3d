import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)
GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def engine_lib():
    """Builds (if needed) and loads the CUDA engine library."""
    from qsource_gb300 import abi, build
    build.build()
    return abi.load_library()


@pytest.fixture(scope="session")
def golden():
    import json
    with open(os.path.join(GOLDEN, "golden.json")) as f:
        return json.load(f)


def golden_system(name):
    from qsource_gb300.system import System
    return System.load_npz(os.path.join(GOLDEN, f"{name}.npz"))
