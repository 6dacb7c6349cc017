import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "gpu-stream-join-benchmark_gb300")
for p in (PKG, os.path.join(ROOT, "oracle"), os.path.join(ROOT, "tests")):
    if p not in sys.path:
        sys.path.insert(0, p)

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the library's kernels)")


@pytest.fixture(scope="session")
def oracle():
    import oracle_py

    oracle_py.build()
    return oracle_py


@pytest.fixture(scope="session")
def lib():
    """The CUDA library, built in-tree (fails loudly if it cannot be built)."""
    import build as b

    b.build_lib()
    import sjbg

    sjbg.load()
    return sjbg


@pytest.fixture(scope="session")
def harness():
    """Path of the C++ runExperiment harness, built in-tree over the library."""
    import build as b

    b.build_lib()
    return b.build_harness()


@pytest.fixture(scope="session")
def golden():
    import json

    with open(os.path.join(GOLDEN, "golden.json")) as f:
        return json.load(f)
