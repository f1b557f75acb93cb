import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden")
REFERENCE = os.environ.get("PHYLOCSF_REFERENCE", "/root/reference")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a GB300 (sm_103a) GPU")
    config.addinivalue_line("markers", "slow: long-running oracle case")


@pytest.fixture(scope="session")
def reference_dir():
    if not os.path.isdir(os.path.join(REFERENCE, "PhyloCSF_Parameters")):
        pytest.skip("reference source tree not available")
    return REFERENCE
