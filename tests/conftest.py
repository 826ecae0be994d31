import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


def _has_gpu():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


HAS_GPU = _has_gpu()


def pytest_collection_modifyitems(config, items):
    if HAS_GPU:
        return
    skip = pytest.mark.skip(reason="no CUDA GPU on this host")
    for it in items:
        if "gpu" in it.keywords:
            it.add_marker(skip)


@pytest.fixture(scope="session")
def oracle_lib():
    """The CPU restatement of the reference (test infrastructure only)."""
    import oracle
    try:
        o = oracle.Oracle()
    except RuntimeError as exc:
        pytest.skip("oracle unavailable: %s" % exc)
    o.set_threads(min(8, os.cpu_count() or 1))
    return o


@pytest.fixture(scope="session")
def hq():
    """The product library (built in-tree)."""
    import hqrrp_gb300
    hqrrp_gb300.build()
    hqrrp_gb300.load()
    return hqrrp_gb300
