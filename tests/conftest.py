"""Test configuration: the `gpu` marker and import paths.

`-m "not gpu"` runs on a CPU-only host: the oracle against the golden
fixtures, host logic, and that the C-ABI library loads and exports every
symbol include/*.h declares.  `-m gpu` runs the parity tests proper on a GPU,
through the C ABI.
"""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "ipdps15-pattern_gb300")
for p in (ROOT, PKG, os.path.join(ROOT, "tests")):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (run with -m gpu)")
    config.addinivalue_line("markers", "slow: takes more than a few seconds on CPU")


@pytest.fixture(scope="session")
def built_lib():
    """Builds the CUDA library (sm_103a) if it is missing, then loads it."""
    import build as pkg_build  # ipdps15-pattern_gb300/build.py
    import irregular_gb300 as irr
    if not os.path.exists(irr.LIB_PATH):
        pkg_build.build()
    return irr.load()


@pytest.fixture(scope="session")
def oracle_lib():
    from oracle import oracle as O
    O.build()
    return O
