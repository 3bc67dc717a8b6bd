"""Shared test setup.

* registers the ``gpu`` marker (tests that need a CUDA device);
* puts the repository root (oracle package, bench) and the library package
  directory (qp3d, synthetic) on sys.path;
* builds the library and the oracle once per session if they are missing.
"""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "gpu-c_3dqmodeling_gb300")
for p in (ROOT, PKG):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300)")


@pytest.fixture(scope="session", autouse=True)
def _built():
    import build as pkg_build          # gpu-c_3dqmodeling_gb300/build.py
    from oracle import build as oracle_build
    pkg_build.build()
    oracle_build.build_oracle()
    yield


@pytest.fixture(scope="session")
def ctx():
    import qp3d
    c = qp3d.Context(0)
    yield c
    c.close()
