"""Shared test setup: import paths, the `gpu` marker and device detection."""
import os
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
PKG_ROOT = ROOT / "itensornumericalanalysis.jl_gb300"
for p in (str(ROOT), str(PKG_ROOT)):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device and the built libtnfa.so")


def _has_gpu() -> bool:
    try:
        import torch

        return torch.cuda.is_available()
    except Exception:
        return False


HAS_GPU = _has_gpu()


def pytest_collection_modifyitems(config, items):
    if HAS_GPU:
        return
    skip = pytest.mark.skip(reason="no CUDA device")
    for item in items:
        if "gpu" in item.keywords:
            item.add_marker(skip)


@pytest.fixture(scope="session")
def ina():
    """The product package with its library loaded (GPU tests only)."""
    import itensornumericalanalysis as m
    from itensornumericalanalysis import _build

    if not _build.LIB_PATH.exists():
        _build.build()
    m._lib.load()
    return m
