"""Shared test configuration.

Markers: `gpu` tests need a CUDA device and the built libiegpu.so; everything
else runs on the CPU.  Paths to the package, the oracle and the golden
fixtures are put on sys.path here.
"""
from __future__ import annotations

import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
PKG = ROOT / "inflation-easy_gb300"
ORACLE = ROOT / "oracle"
GOLDEN = ROOT / "tests" / "golden"
INPUTS = GOLDEN / "inputs"

for p in (str(PKG), str(ORACLE), str(ROOT)):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU and the built engine")


@pytest.fixture(scope="session")
def oracle_mod():
    import ieo
    ieo.build()
    return ieo


@pytest.fixture(scope="session")
def tables():
    import numpy as np
    return tuple(np.loadtxt(INPUTS / n) for n in ("field_values.dat", "potential.dat", "potential_derivative.dat"))


@pytest.fixture(scope="session")
def engine():
    """The engine binding; building it is the job of __graft_entry__.build()."""
    import iegpu
    iegpu.load()
    return iegpu
