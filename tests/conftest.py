"""Shared pytest configuration.

``gpu``: needs a CUDA device (GB300) and the built ``libgato_cuda`` library.
Everything else runs on the CPU: the oracle against the reference's own
known-answer invariants, host-side logic, and the C-ABI export table.
"""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: requires a CUDA GPU and the built CUDA library")
    config.addinivalue_line("markers", "slow: long-running CPU check")


def pytest_collection_modifyitems(config, items):
    # Files named test_zz_* run last so a stop-at-first-failure run has
    # already exercised everything else.
    items.sort(key=lambda it: os.path.basename(str(it.fspath)).startswith("test_zz_"))
