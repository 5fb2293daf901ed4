import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "matrix-free-dealii-precice_gb300")
for p in (ROOT, PKG, os.path.join(ROOT, "oracle")):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: test needs a CUDA GPU (GB300)")


@pytest.fixture(scope="session")
def ctx():
    import torch
    import build as pkg_build
    import mfgpu
    pkg_build.build()
    torch.cuda.init()
    c = mfgpu.Context(0)
    yield c
    c.close()
