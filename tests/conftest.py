import json
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def golden():
    with open(os.path.join(ROOT, "tests", "golden", "reference_known_answers.json")) as f:
        return json.load(f)


@pytest.fixture(scope="session")
def O():
    from oracle import pn_oracle
    return pn_oracle


@pytest.fixture(scope="session")
def pkg():
    import __graft_entry__
    return __graft_entry__.package()


def jfloat(v, dtype=float):
    """Decode the fixture's float encoding ("inf", "nan", ["prev"/"next", v])."""
    import numpy as np
    if isinstance(v, str):
        return dtype(float(v))
    if isinstance(v, list):
        kind, base = v
        b = dtype(base)
        return np.nextafter(b, dtype(-np.inf) if kind == "prev" else dtype(np.inf))
    return dtype(v)
