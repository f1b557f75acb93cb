import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden")
# the mlin/PhyloCSF source tree, for the tests that read its files directly (skipped without it)
REFERENCE = os.environ.get("PHYLOCSF_REFERENCE", "")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a GB300 (sm_103a) GPU")
    config.addinivalue_line("markers", "slow: long-running oracle case")


@pytest.fixture(scope="session")
def reference_dir():
    if not REFERENCE or not os.path.isdir(os.path.join(REFERENCE, "PhyloCSF_Parameters")):
        pytest.skip("PHYLOCSF_REFERENCE does not name the reference source tree")
    return REFERENCE
