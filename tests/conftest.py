"""Shared pytest configuration.

Tests marked ``gpu`` need a GB300 (they call the CUDA library through its
C-ABI); everything else runs on the CPU.  The oracle (oracle/) is test
infrastructure: tests import it only as the checker.
"""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (ROOT, os.path.join(ROOT, "oracle")):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")
