import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

# Tests that read the reference's own files (its meshes, the line ranges of its
# sources) find the checkout through PHYBS_REFERENCE; where this machine has one
# at the usual place it is the default.  Elsewhere those tests skip.
if not os.environ.get("PHYBS_REFERENCE") and os.path.isdir("/root/reference/FVM"):
    os.environ["PHYBS_REFERENCE"] = "/root/reference"


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a GB300 (sm_103) and the built CUDA library")
