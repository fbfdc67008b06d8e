"""Shared pytest setup: import paths, the `gpu` marker, and session fixtures
for the CUDA library and the CPU oracle (the parity checker)."""
import os
import sys

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(REPO, "ns-lsm-single-phase_gb300")
for p in (REPO, PKG, os.path.join(REPO, "oracle"), os.path.join(REPO, "tests")):
    if p not in sys.path:
        sys.path.insert(0, p)


def _cuda_available() -> bool:
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300)")


def pytest_collection_modifyitems(config, items):
    if _cuda_available():
        return
    skip = pytest.mark.skip(reason="no CUDA device")
    for it in items:
        if "gpu" in it.keywords:
            it.add_marker(skip)


@pytest.fixture(scope="session")
def oracle():
    import oracle as O
    O.build()
    return O.Oracle()


@pytest.fixture(scope="session")
def lib_built():
    from nslsm.build import build
    return build()


@pytest.fixture(scope="session")
def ls(lib_built):
    from nslsm import LevelSet
    h = LevelSet(device=0)
    yield h
    h.close()
