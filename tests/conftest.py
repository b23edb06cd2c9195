import os
import sys

import pytest

# tests start from the built-in stage-kernel defaults, not from an autotune cache on this machine
# (the cache test points the variable at a file of its own)
os.environ["ATSAT_DYN_TUNE_CACHE"] = "off"

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
TESTS = os.path.dirname(os.path.abspath(__file__))
for _p in (ROOT, TESTS):
    if _p not in sys.path:
        sys.path.insert(0, _p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a) and the built library")
    config.addinivalue_line("markers", "slow: full-size grids; minutes on the CPU")
