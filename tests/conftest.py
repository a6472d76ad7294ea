"""Shared test setup.

* `-m "not gpu"` (CPU): the oracle against the reference's golden vectors,
  host logic (checkpoint format, generators, serving scheduler), and the
  C-ABI library's symbol table.  No CUDA compute runs.
* `-m gpu`: parity of the CUDA path (through the C ABI) against the oracle.
"""
from __future__ import annotations

import os
import sys

import numpy as np
import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG_DIR = os.path.join(REPO, "nbody-gpu-sim_gb300")
for p in (REPO, PKG_DIR):
    if p not in sys.path:
        sys.path.insert(0, p)

GOLDEN = os.path.join(REPO, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the sm_103a library)")
    config.addinivalue_line("markers", "slow: long-running case")


@pytest.fixture(scope="session")
def orc():
    from oracle.oracle import Oracle
    return Oracle()


@pytest.fixture(scope="session")
def golden():
    def load(name):
        return np.load(os.path.join(GOLDEN, name))
    return load


@pytest.fixture(scope="session")
def nb():
    import nbgb
    nbgb.lib()  # builds if needed, fails loudly if the library cannot load
    return nbgb


def rel_err(a, b, floor=0.0):
    """|a-b| / max(|b|, floor), componentwise on (n,3) or vector-norm rows."""
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return np.abs(a - b) / np.maximum(np.abs(b), floor)


def vec_rel_err(ax, ay, az, bx, by, bz):
    """Per-target |a - b| / |b| with vector norms (force error metric)."""
    a = np.stack([ax, ay, az], 1).astype(np.float64)
    b = np.stack([bx, by, bz], 1).astype(np.float64)
    nb = np.linalg.norm(b, axis=1)
    return np.linalg.norm(a - b, axis=1) / np.maximum(nb, 1e-300)
