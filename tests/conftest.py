import gzip
import json
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300)")


def golden(name):
    with gzip.open(os.path.join(GOLDEN, name + ".json.gz"), "rt") as f:
        return json.load(f)


@pytest.fixture(scope="session")
def oracle_lib():
    import oracle
    return oracle.load()


@pytest.fixture(scope="session")
def m8():
    from phonomc_gb300 import synthetic
    return synthetic.make_material(mesh=8)


@pytest.fixture(scope="session")
def m8c():
    from phonomc_gb300 import synthetic
    return synthetic.make_material(mesh=8, callaway=True)


def rel_close(a, b, rtol, atol=0.0):
    a = np.asarray(a, dtype=float)
    b = np.asarray(b, dtype=float)
    return np.allclose(a, b, rtol=rtol, atol=atol, equal_nan=True)
