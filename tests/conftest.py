"""Shared test set-up: import paths and the `gpu` marker.

`-m "not gpu"` runs the oracle checks, host logic and C-ABI export checks on
the CPU; `-m gpu` runs the CUDA parity tests (they call the library through
its C ABI and compare with the oracle).
"""
import os
import sys

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (REPO, os.path.join(REPO, "vfs-wind_gb300"), os.path.join(REPO, "oracle")):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


def _cuda_available():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


def pytest_collection_modifyitems(config, items):
    if _cuda_available():
        return
    skip = pytest.mark.skip(reason="no CUDA device")
    for it in items:
        if "gpu" in it.keywords:
            it.add_marker(skip)


@pytest.fixture(scope="session")
def cuda_lib():
    from vfs_poisson import _build
    _build.build()
    import vfs_poisson
    return vfs_poisson.load()
