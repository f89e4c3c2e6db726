import json
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (ROOT, os.path.join(ROOT, "oracle"), os.path.dirname(os.path.abspath(__file__))):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def oracle():
    import oracle as O

    O.build()
    return O


@pytest.fixture(scope="session")
def zc():
    """The CUDA backend package, with the in-tree library built."""
    from zeno_gb300 import backend, build

    build.build()
    backend.load()
    return backend


@pytest.fixture(scope="session")
def examples():
    with open(os.path.join(ROOT, "tests", "golden", "examples.json")) as f:
        return json.load(f)
