"""Shared fixtures: the product library (nprsph), the CPU oracle, and the gpu marker."""
from __future__ import annotations

import importlib
import sys
from pathlib import Path

import pytest

REPO = Path(__file__).resolve().parent.parent
PKG = REPO / "npr-sph_gb300"
for p in (str(PKG), str(REPO)):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs on the GB300 box)")


def _ensure_built():
    import build as pkg_build  # npr-sph_gb300/build.py

    pkg_build.build()
    from oracle import oracle as orc

    if not orc.LIB.exists():
        orc.build(with_ref=True)


_ensure_built()


@pytest.fixture(scope="session")
def sph():
    return importlib.import_module("nprsph")


@pytest.fixture(scope="session")
def orc():
    from oracle import oracle as o

    return o


def cuda_ok() -> bool:
    try:
        import torch

        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.fixture(scope="session")
def gpu():
    if not cuda_ok():
        pytest.fail("this test needs a CUDA GPU (run with -m 'not gpu' on a machine without one)")
    import torch

    torch.cuda.init()
    return torch.device("cuda:0")
