"""pytest configuration: the `gpu` marker and shared small model fixtures."""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


def has_gpu() -> bool:
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


# The reference checkout, read as text or imported by CPU tests only (it is
# not present where the GPU tests run).  PQMC_REFERENCE overrides the
# location; tests that need it skip when it is absent.
REFERENCE_ROOT = os.environ.get("PQMC_REFERENCE", "/root/reference")


@pytest.fixture
def reference_root():
    if not os.path.isdir(REFERENCE_ROOT):
        pytest.skip("reference checkout not present")
    return REFERENCE_ROOT
