import gzip
import json
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300)")


def load_golden(name):
    with gzip.open(os.path.join(GOLDEN, name), "rt") as f:
        return [json.loads(line) for line in f]


@pytest.fixture(scope="session")
def wfa_golden():
    return load_golden("wfa_golden.json.gz")


@pytest.fixture(scope="session")
def sw_golden():
    return load_golden("sw_golden.json.gz")


@pytest.fixture(scope="session")
def real_golden():
    return load_golden("real_golden.json.gz")
