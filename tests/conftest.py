import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the compiled sm_103a library")
    config.addinivalue_line("markers", "slow: full-size (2^28) workloads")


def pytest_collection_modifyitems(config, items):
    import torch

    if torch.cuda.is_available():
        return
    skip = pytest.mark.skip(reason="no CUDA device")
    for item in items:
        if "gpu" in item.keywords:
            item.add_marker(skip)


@pytest.fixture(scope="session")
def gms_lib():
    """The compiled library (built on first use, e.g. on a fresh GPU machine)."""
    from gpumultisplit_gb300 import build as gbuild

    gbuild.build()
    import gpumultisplit_gb300 as gms

    return gms.load()


@pytest.fixture(scope="session")
def oracle_mod():
    import oracle

    if not oracle.LIB.exists():
        oracle.build(with_ref=False)
    return oracle


@pytest.fixture(scope="session")
def golden():
    import json

    with open(os.path.join(ROOT, "tests", "golden", "golden.json")) as f:
        return json.load(f)["cases"]
