"""Shared test setup.

Markers: `gpu` = needs a CUDA device and liblgca_gpu.so (run with -m gpu on a
GB300); everything else runs on the CPU.  The oracle (oracle/) is the
checker: tests compare the GPU path against it and against the golden
fixtures in tests/golden/, generated from the reference itself.
"""
import json
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)
GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU and the built liblgca_gpu.so")
    config.addinivalue_line("markers", "slow: full-size workload checks (minutes)")


@pytest.fixture(scope="session")
def oracle():
    from oracle import oracle as O
    O.build(ref=False)
    return O


@pytest.fixture(scope="session")
def ref(oracle):
    """The compiled reference harness (only where the reference sources are)."""
    if not os.path.isdir(os.path.join(oracle.REFERENCE_DIR, "src")) and not oracle.ref_available():
        pytest.skip("reference sources not present on this machine")
    oracle.build(ref=True)
    return oracle


@pytest.fixture(scope="session")
def gpu():
    """The CUDA library, built for sm_103a; fails loudly if it cannot load."""
    import lgca_gb300
    lgca_gb300.build()
    lib = lgca_gb300.lib()
    assert lib.lgca_abi_version() == 1
    return lgca_gb300


def load_npz(name):
    return np.load(os.path.join(GOLDEN, name))


def load_json(name):
    with open(os.path.join(GOLDEN, name)) as f:
        return json.load(f)
