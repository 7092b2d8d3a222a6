import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden")
# the reference checkout, named by WHALE_REFERENCE_DIR where the fixtures are
# regenerated or re-checked against it (unset elsewhere: those tests skip)
REFERENCE = os.environ.get("WHALE_REFERENCE_DIR", "")

sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the sm_103a kernels)")


@pytest.fixture(scope="session")
def W():
    import __graft_entry__

    return __graft_entry__.load_package()


@pytest.fixture(scope="session")
def O():
    import oracle

    oracle.build()
    return oracle


def read(path):
    with open(path) as fh:
        return fh.read()


@pytest.fixture(scope="session")
def ex1_tree():
    return read(os.path.join(GOLDEN, "example1_tree.nw")).strip()


@pytest.fixture(scope="session")
def ex1_files():
    d = os.path.join(GOLDEN, "example1")
    return [os.path.join(d, f) for f in sorted(os.listdir(d)) if f.endswith(".ale")]


@pytest.fixture(scope="session")
def golden():
    import json

    with open(os.path.join(GOLDEN, "golden.json")) as fh:
        return json.load(fh)
