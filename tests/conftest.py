"""Shared test setup.

Tests marked ``gpu`` need a CUDA GPU and the built te_gpu library; every other
test runs on the CPU.  The oracle (oracle/, a CPU restatement of the
reference, test infrastructure only) is built on first use.
"""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (ROOT, os.path.join(ROOT, "oracle")):
    if p not in sys.path:
        sys.path.insert(0, p)

def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (run with -m gpu)")


@pytest.fixture(scope="session")
def oracle():
    import oracle as orc

    orc.build()
    return orc.Oracle("teo")


@pytest.fixture(scope="session")
def ref():
    """ThunderEgg itself, compiled from its sources (only where they exist)."""
    import oracle as orc

    if not orc.ref_sources_present():
        pytest.skip("reference sources not present")
    orc.build(ref=True)
    return orc.Oracle("teref")


@pytest.fixture(scope="session")
def te():
    import thunderegg_gb300
    from thunderegg_gb300 import build

    build.build()
    return thunderegg_gb300


def rel_err(a, b):
    """max |a - b| / max |b| (infinity-norm relative error)."""
    import numpy as np

    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    scale = max(float(np.abs(b).max()), 1e-300)
    return float(np.abs(a - b).max()) / scale
