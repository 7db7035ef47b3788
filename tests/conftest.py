"""Test configuration: the `gpu` marker and one-time builds of the oracle and
the library (in-tree, no install)."""
import os
import subprocess
import sys

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
for p in (HERE, ROOT, os.path.join(ROOT, "bm4d-of_gb300"), os.path.join(ROOT, "oracle")):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def oracle():
    import pyoracle
    pyoracle.build()
    return pyoracle.Oracle()


@pytest.fixture(scope="session")
def reference():
    import pyoracle
    pyoracle.build()
    if not pyoracle.Reference.available():
        pytest.skip("reference sources not present (oracle/_ref not built)")
    return pyoracle.Reference()


@pytest.fixture(scope="session")
def gpulib():
    import build as pkgbuild
    pkgbuild.build()
    import bm4dof
    return bm4dof


@pytest.fixture(scope="session")
def gpuctx(gpulib):
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    ctx = gpulib.Context(0)
    yield ctx
    ctx.close()
