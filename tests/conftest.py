import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (run with -m gpu)")
    config.addinivalue_line("markers", "slow: long-running")


@pytest.fixture(autouse=True)
def _fresh_bc_registry():
    """BC ids are process-global and never reused (as in XLB); start each test at 1."""
    from xlb_gb300.operator.boundary_condition import boundary_condition_registry

    boundary_condition_registry.id_to_bc.clear()
    boundary_condition_registry.bc_to_id.clear()
    boundary_condition_registry.next_id = 1
    yield


def pytest_collection_modifyitems(config, items):
    try:
        import torch

        has_gpu = torch.cuda.is_available()
    except Exception:
        has_gpu = False
    if has_gpu:
        return
    skip = pytest.mark.skip(reason="no CUDA GPU in this environment")
    for item in items:
        if "gpu" in item.keywords:
            item.add_marker(skip)
