import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (run with -m gpu)")


@pytest.fixture(scope="session")
def port():
    import pyoracle as po

    po.build_port()
    return po.Oracle("port")


@pytest.fixture(scope="session")
def ref():
    """The reference's own code (x86-64 hosts with the reference tree only)."""
    import pyoracle as po

    try:
        lib = po.build_ref()
    except Exception as e:  # build failure is a skip, not an error: it is the checker's checker
        pytest.skip(f"reference harness did not build: {e}")
    if lib is None:
        pytest.skip("reference tree not present on this host")
    return po.Oracle("ref")


@pytest.fixture(scope="session")
def golden():
    import numpy as np

    d = os.path.join(ROOT, "tests", "golden")
    return {k: np.load(os.path.join(d, f"{k}.npz")) for k in ("primitives", "bvh", "scenes")}


@pytest.fixture(scope="session")
def gpu_lib():
    """The GB300 library, built in-tree; GPU tests fail loudly without it."""
    import torch

    if not torch.cuda.is_available():
        pytest.fail("-m gpu tests need a CUDA device")
    from vk_cinematic_gb300 import gbsp

    return gbsp.load()
