"""Shared fixtures.  `-m "not gpu"` runs the oracle, host logic and ABI checks
on the CPU; `-m gpu` runs the parity tests of the CUDA path through the C ABI.
"""
from __future__ import annotations

import sys
from pathlib import Path

import pytest

REPO = Path(__file__).resolve().parent.parent
PKG = REPO / "build-up-phase_gb300"
for p in (str(REPO), str(PKG)):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def rtlib():
    """librtcore.so, built in-tree if a source is newer (nvcc only, no GPU)."""
    import build as rt_build  # build-up-phase_gb300/build.py
    rt_build.build()
    import rtcore
    return rtcore.load()


@pytest.fixture(scope="session")
def orc():
    import oracle
    oracle.build()
    oracle.load()
    return oracle


@pytest.fixture(scope="session")
def ctx(rtlib):
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import rtcore
    c = rtcore.Context(0)
    yield c
    c.close()
