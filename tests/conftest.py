"""Shared test set-up: marker registration and import paths.

CPU tests (-m "not gpu") exercise the oracle against analytic known answers,
the host-side C-ABI helpers and the multi-rank host logic.  GPU tests
(-m gpu) call the CUDA library through the C-ABI and compare with the oracle.
"""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "pimd-tunneling_gb300")
for p in (os.path.join(PKG, "python"), os.path.join(ROOT, "oracle"), PKG, ROOT):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def oracle():
    import oracle as O
    O.lib()
    return O


@pytest.fixture(scope="session")
def pg():
    import build as B
    B.build()
    import pimdgpu
    pimdgpu.lib()
    return pimdgpu


@pytest.fixture(scope="session")
def ctx(pg):
    c = pg.Context(0)
    yield c
    c.close()
