import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "bwa-mem4_gb300")
for p in (ROOT, PKG, os.path.dirname(os.path.abspath(__file__))):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs on the GB300 box)")


@pytest.fixture(scope="session")
def built():
    """Build libbwacuda.so / libbwasynth.so / the oracle once per session."""
    import importlib.util

    import oracle

    spec = importlib.util.spec_from_file_location("bwacuda_build", os.path.join(PKG, "build.py"))
    B = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(B)
    B.build()
    oracle.build()
    return True


@pytest.fixture(scope="session")
def ctx(built):
    import torch

    if not torch.cuda.is_available():
        pytest.fail("a GPU test ran without a visible CUDA device")
    import bwacuda

    c = bwacuda.Context(0)
    yield c
    c.close()
