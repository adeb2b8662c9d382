"""Shared test setup.

`gpu`-marked tests need a GB300 (CUDA) and call the CUDA library through its
C ABI; everything else runs on CPU (oracle, host utilities, library exports).
"""

import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "parallel-correlation-clustering_gb300")
for p in (PKG, os.path.join(ROOT, "oracle"), ROOT):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def built():
    """Builds the native libraries (and the oracle) once per session."""
    import build_native
    import oracle
    build_native.build_all()
    oracle.build()
    return True


@pytest.fixture(scope="session")
def ctx(built):
    import pcc_gb300
    c = pcc_gb300.Context(0)
    yield c
    c.close()


def rand_state(n, nclusters, seed, node_weights=None):
    """A consistent (C, s, k, K) clustering state with random labels."""
    rng = np.random.default_rng(seed)
    C = rng.integers(0, max(1, nclusters), size=n).astype(np.uint32)
    k = np.ones(n) if node_weights is None else np.asarray(node_weights, np.float64)
    s = np.bincount(C, minlength=n).astype(np.uint32)
    K = np.bincount(C, weights=k, minlength=n).astype(np.float64)
    return C, s, k, K
